"""Benchmark of the GB300 FMM RK4 step (one JSON line on stdout).

Workload (headline): Plummer sphere of 4,194,304 equal-mass particles (G = 1,
M = 1, scale radius 1; radii by inverse CDF r = (u^(-2/3) - 1)^(-1/2) with
r <= 10, isotropic directions, speeds by von Neumann rejection from the
Plummer distribution function; seed 2), eps = 0.005, p = 8, s = 64, mixed
precision with the workload's BF16 hi/lo tensor-core M2L split (--m2l tf32
for the library's default 3 x TF32 split), RK4 dt = 5e-4. A step is one RK4
step (four force evaluations, tree rebuilt at every stage).

  value   particle-steps/s with the state resident in HBM (CUDA events on the
          solver's stream around exactly --steps steps)
  e2e     the same through the C-ABI with host buffers: per step, upload of
          x, v from pinned host memory, one RK4 step, download of x, v
  plain_fp64  the same step with every stage in FP64 (the plain form)
  accurate  the accurate mode (far field times G plus the softening
          correction) at p = 10: the mixed form and the plain FP64 form, both
          timed over the same steps, with their errors against the FP64 direct
          sum and mixed_over_plain
  m2l_other_split  the same step with the other M2L split (value, energy drift)
  batched  512 independent Plummer systems of uneven N (one batch step)
  cpu_baseline  the reference's algorithm on the host cores (oracle port, or
          the compiled reference where it exists), on a bounded sample of one
          force evaluation, extrapolated to a step

``--workload clustered`` runs the adaptive-depth stress workload instead:
16,777,216 particles in 8 equal-mass Plummer clusters (scale radii uniform in
[0.01, 0.1], centres uniform in [0, 1)^3, Gaussian bulk velocities sigma 0.3)
plus a 5% uniform background, eps = 1e-4, p = 8, s = 64, dt = 1e-4, seed 4.
``--workload uniform``: 1,048,576 equal-mass particles uniform in the unit
cube at rest, eps = 1e-3, p = 6, s = 64, dt = 1e-4, seed 1.

``--impl reference`` times the reference's CPU implementation instead
(same metric and config) and prints its own line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

# many concurrent streams in the batching form: one hardware queue each (set before CUDA starts)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
# the library's GB300 tuning cache (vipp_gb300.autotune's measured entries),
# applied at upload unless the caller names another file or --no-tuning-cache
SHIPPED_TUNING = os.path.join(os.path.dirname(os.path.abspath(__file__)), "vipp-nbody-bench_gb300", "vipp_gb300",
                              "tuning_gb300.txt")

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "vipp-nbody-bench_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from vipp_gb300.workloads import clustered, plummer, uniform  # noqa: E402  (numpy only; the library loads later)

METRIC = "RK4 particle-steps/s at stated FP64-direct force error; mixed/batched vs plain"
UNIT = "particle-steps/s"
FP32_LANES_PER_SM = 128


def make_workload(args, rank=0, device=None):
    """(x, v, seed, name) of the selected workload; replicas use seed + rank.
    With a device, the clustered workload is drawn there (gb_init_clustered)
    and copied back; otherwise on the host (workloads.clustered: the same
    distribution, other numbers)."""
    if args.workload == "clustered":
        seed = 4 + rank
        if device is not None:
            import vipp_gb300
            with vipp_gb300.Solver(p=4, s=args.s, eps=args.eps, m=1.0 / args.n, device=device) as g:
                g.init_clustered(args.n, seed)
                x, v = g.postprocess()
            return x, v, seed, f"clustered-{args.n} (8 Plummer clusters + 5% background, drawn on the GPU)"
        x, v, _ = clustered(args.n, seed)
        return x, v, seed, f"clustered-{args.n} (8 Plummer clusters + 5% background)"
    if args.workload == "uniform":
        seed = 1 + rank
        x, v = uniform(args.n, seed)
        return x, v, seed, f"uniform-{args.n} (unit cube, at rest)"
    seed = 2 + rank
    x, v = plummer(args.n, seed)
    return x, v, seed, f"plummer-{args.n}"


# DRAM bytes (read + write) per launch of the BF16-split M2L on the 4M
# workload, from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum)
M2L_BF16_TRAFFIC = 135549184 + 14860544


def batch_measure(steps=50, warmup=2, nsys=512, seed=3, sample=32, flags=0, form="forest", rank=0, ws=1, device=0):
    """Batching form: nsys Plummer systems, N log-uniform in [1024, 65536],
    scale radius uniform in [0.5, 2] (positions x R, velocities x R^-1/2), total
    mass 1 each, eps = 0.01, p = 6, s = 32, mixed precision, dt = 1e-3, all
    advanced together (gb_batch_rk4_step). form "forest": one context, one
    launch per kernel class over all systems; "contexts": one context and step
    graph per system. Wall clock per step (a batch step returns after every
    system's step has finished); error vs the FP64 direct sum on `sample`
    systems. With ws > 1 ranks the systems are split into contiguous runs of
    about equal particle count (vipp_gb300.shard_systems), each rank runs its
    run as one batch (the same systems the whole batch draws), and the timed
    steps are bracketed by barriers, max over ranks; errors come from rank 0's
    systems."""
    import vipp_gb300
    rng = np.random.default_rng(seed)
    sizes_all = np.rint(np.exp(rng.uniform(math.log(1024), math.log(65536), nsys))).astype(np.int64)
    first, last = vipp_gb300.shard_systems(sizes_all, ws)[rank]
    sizes = sizes_all[first:last]
    nsys = len(sizes)
    if form == "contexts":
        flags |= vipp_gb300.FLAG_BATCH_CONTEXTS
    t0 = time.perf_counter()
    b = vipp_gb300.Batch(sizes, p=6, s=32, eps=0.01, masses=1.0 / sizes, precision="mixed", flags=flags, device=device)
    b.init_plummer(seed=seed, r_lo=0.5, r_hi=2.0, first=first)  # every system drawn on the GPU
    setup = time.perf_counter() - t0
    for _ in range(warmup):
        b.step(1e-3)
    l0 = b.launch_count()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(steps):
        b.step(1e-3)
    dt_wall = max_over_ranks(time.perf_counter() - t0, ws)
    launches = (b.launch_count() - l0) / steps
    st = b.stats()
    errs = []
    xb, _ = b.download()
    acc = b.accel() if b.forest else None
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k in (np.linspace(0, nsys - 1, sample).astype(int) if rank == 0 and nsys else []):
        a = acc[off[k]:off[k + 1]] if acc is not None else b.system_accel(int(k))
        with vipp_gb300.Solver(p=6, s=32, eps=0.01, m=1.0 / sizes[k], precision="fp64", device=device) as sd:
            sd.preprocess(xb[off[k]:off[k + 1]], np.zeros((sizes[k], 3)))
            ad = sd.direct_accel()
        e = np.linalg.norm(a - ad, axis=1) / np.linalg.norm(ad, axis=1)
        errs.append(float(math.sqrt(np.mean(e * e))))
    b.close()
    n = int(sizes_all.sum())
    return {"workload": f"{len(sizes_all)} Plummer systems, N log-uniform in [1024, 65536] (seed {seed}), R in [0.5, 2] "
                        "(systems drawn on the GPU), p=6 s=32 eps=0.01 mixed, dt=1e-3", "form": form,
            "value": n * steps / dt_wall, "unit": UNIT, "n_total": n, "n_gpus": ws,
            "scaling": "strong (the 512 systems split over the ranks)" if ws > 1 else None,
            "systems": len(sizes_all), "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * dt_wall / steps,
            "launches_per_step": launches, "tree": {k: st[k] for k in ("ncells", "nleaves", "depth", "m2l_pairs",
                                                                        "p2p_pairs")},
            "setup_s": setup, "rms_rel_err_vs_fp64_direct_per_system": errs,
            "timing": "host wall clock per gb_batch_rk4_step (it returns after all systems' steps)"}


def timed_steps(sol, steps, dt, local):
    """Seconds of exactly `steps` RK4 steps by CUDA events on the solver's stream."""
    import torch
    st = torch.cuda.ExternalStream(sol.stream_ptr(), device=local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sol.sync()
    e0.record(st)
    for _ in range(steps):
        sol.solve(dt)
    e1.record(st)
    e1.synchronize()
    sol.sync()
    return e0.elapsed_time(e1) / 1e3


def accurate_measure(x, v, args, local, tg, ad):
    """The accurate mode (GB_MODE_ACCURATE: far field times G plus the
    softening correction) on the same workload at p = args.acc_p: the mixed
    form (3 x TF32 M2L split unless --acc-m2l bf16) and the plain all-FP64
    form, both timed by CUDA events over the same args.acc_steps steps after
    one untimed step, both checked against the FP64 direct sum on the same
    sample (tg, ad)."""
    import vipp_gb300
    n = x.shape[0]
    m = 1.0 / n
    out = {"p": args.acc_p, "mode": "accurate", "steps": args.acc_steps}
    forms = (("mixed", vipp_gb300.FLAG_M2L_BF16 if args.acc_m2l == "bf16" else 0), ("fp64", 0))
    for prec, flags in forms:
        with vipp_gb300.Solver(p=args.acc_p, s=args.s, eps=args.eps, G=1.0, m=m, precision=prec, device=local,
                               flags=flags, mode="accurate") as sa:
            sa.preprocess(x, v)
            tun = sa.tuning()
            a = sa.accel()
            e = np.linalg.norm(a[tg] - ad, axis=1) / np.linalg.norm(ad, axis=1)
            sa.solve(args.dt)  # captures the step graph
            c0 = sa.conserved() if (prec == "mixed" and not args.no_energy) else None
            t = timed_steps(sa, args.acc_steps, args.dt, local)
            drift = None
            if c0 is not None:
                c1 = sa.conserved()
                drift = abs(c1["total"] - c0["total"]) / abs(c0["total"])
            kt = None
            if prec == "mixed":
                sa.enable_timing(True)
                sa.kernel_times()
                sa.solve(args.dt)
                sa.sync()
                kt = {k: round(val[0], 4) for k, val in sa.kernel_times().items()}
                sa.enable_timing(False)
        out[prec] = {"value": n * args.acc_steps / t, "unit": UNIT, "ms_per_step": 1e3 * t / args.acc_steps,
                     "rms_rel_err_vs_fp64_direct": float(math.sqrt(np.mean(e * e))),
                     "max_rel_err_vs_fp64_direct": float(e.max()), "error_sample": int(len(tg)),
                     "m2l_split": ("bf16 hi/lo" if flags else "3 x tf32") if prec == "mixed" else "fp64 cuda cores",
                     "timing": f"CUDA events around {args.acc_steps} steps on the solver's stream", "tuning": tun}
        if drift is not None:
            out[prec]["energy_rel_drift"] = drift
            out[prec]["energy_note"] = ("potential of the accurate mode: far field times G with its softening "
                                        "correction, plus the FP64 softened near field")
        if kt:
            out[prec]["kernel_ms_per_step"] = kt
    out["mixed_over_plain"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["both_within_1e-5"] = bool(out["mixed"]["rms_rel_err_vs_fp64_direct"] <= 1e-5
                                   and out["fp64"]["rms_rel_err_vs_fp64_direct"] <= 1e-5)
    return out


class ClockSampler:
    """nvidia-smi samples (every 200 ms) of SM clock and throttle reasons."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for nm, val in zip(names, f[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(val: float, ws: int) -> float:
    if ws <= 1:
        return val
    import torch
    import torch.distributed as dist

    t = torch.tensor([val], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def cpu_baseline_sample(x, s, p, eps, target_seconds=12.0):
    """The reference's algorithm (oracle port) on the host cores: the whole
    tree, lists and upward pass of one force evaluation, plus M2L/P2P/L2L/L2P
    of every stride-th cell, scaled up by M2L pair counts."""
    import oracle

    n = x.shape[0]
    stride = 96
    times, counts = oracle.accel_sampled(x, s, 1.0, 1.0 / n, eps, p, stride)
    per_eval = times[0] + times[1] + times[2] * (counts[2] / max(counts[3], 1))
    step = 4 * per_eval
    ref = oracle.ref() is not None and os.environ.get("VIPP_BASELINE_KIND") == "reference"
    return {"value": n / step, "unit": UNIT, "cores": oracle.threads(), "kind": "reference" if ref else "port",
            "sample": (f"one force evaluation of the same {n}-particle workload: full tree+lists "
                       f"({times[0]:.2f} s) and upward pass ({times[1]:.2f} s), far/near work of every "
                       f"{stride}th cell ({int(counts[1])} cells, {times[2]:.2f} s) scaled by M2L pairs "
                       f"{int(counts[2])}/{int(counts[3])}; x4 evaluations per RK4 step"),
            "seconds_per_step_extrapolated": step, "extrapolated": True, "samples": 1}


def run_reference_arm(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    import oracle

    x, v, _, wname = make_workload(args)
    vals = []
    t_start = time.time()
    # CPU runs need no warm-up beyond the first sample; every step is one
    # bounded sample (about 20 s), stopped early to stay within a few minutes
    for k in range(args.steps):
        r = cpu_baseline_sample(x, args.s, args.p, args.eps)
        vals.append(r["value"])
        if time.time() - t_start > 150:
            break
    value = float(np.median(vals))
    cfg = {"workload": f"{wname} p={args.p} s={args.s} eps={args.eps} {args.precision}",
           "N": args.n, "p": args.p, "s": args.s, "eps": args.eps, "dt": args.dt}
    # "steps" counts timed samples: each is one extrapolated RK4 step (4 x one
    # sampled force evaluation), not a run of consecutive steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": len(vals),
            "samples": len(vals), "extrapolated": True,
            "warmup": args.warmup, "ms_per_step": 1e3 * args.n / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"], "extrapolated": True, "samples": len(vals)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    del oracle
    print(json.dumps(line), flush=True)


def parse_args(argv=None):
    """Command line, with the selected workload's defaults filled in: plummer
    N = 4,194,304, eps = 0.005, dt = 5e-4, p = 8; clustered N = 16,777,216,
    eps = 1e-4, dt = 1e-4, p = 8; uniform N = 1,048,576, eps = 1e-3,
    dt = 1e-4, p = 6; s = 64 for all (explicit --n/--eps/--dt/--p win). At
    least 3 warm-up steps on the GPU arm."""
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plummer", choices=["plummer", "clustered", "uniform"],
                    help="plummer: the 4M Plummer sphere (headline); clustered: the 16M adaptive-depth stress "
                         "workload (8 Plummer clusters + 5%% background, eps=1e-4, dt=1e-4); uniform: 1M particles "
                         "in the unit cube at rest (eps=1e-3, p=6, dt=1e-4)")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--p", type=int, default=None)
    ap.add_argument("--s", type=int, default=64)
    ap.add_argument("--eps", type=float, default=None)
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--error-sample", type=int, default=65536)
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 plain-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--flags", type=int, default=0, help="gb_config flags (vipp_gb300.FLAG_*)")
    ap.add_argument("--no-energy", action="store_true", help="skip the total-energy drift (two extra evaluations)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batching form (512 independent systems)")
    ap.add_argument("--batch-steps", type=int, default=50, help="timed steps of the batching form (the configuration's 50)")
    ap.add_argument("--no-contexts", action="store_true",
                    help="skip the batching form's comparison run with one context per system")
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batching form (warm-up --warmup steps, --batch-steps timed) and print its line")
    ap.add_argument("--no-error", action="store_true", help="with --batch-only: skip the per-system error check")
    ap.add_argument("--m2l", default="bf16", choices=["bf16", "tf32"],
                    help="mixed form's tensor-core M2L split: bf16 hi/lo (the 4M Plummer and batching configurations' "
                         "form, GB_FLAG_M2L_BF16) or 3 x tf32 (the library default)")
    ap.add_argument("--no-alt", action="store_true", help="skip the timing of the other M2L split")
    ap.add_argument("--no-accurate", action="store_true", help="skip the accurate-mode line (mixed and plain FP64)")
    ap.add_argument("--tune", action="store_true", help="run the autotuner on the workload; report tuned vs default")
    ap.add_argument("--no-tuning-cache", action="store_true",
                    help="ignore the library's tuning cache (vipp_gb300/tuning_gb300.txt): every line at the defaults")
    ap.add_argument("--tune-out", default=None, help="append the tuned entry to this tuning cache file")
    ap.add_argument("--p2p-occupancy", type=int, default=None, choices=[6, 8],
                    help="override the tuning's mixed P2P kernel build for the main line (registers budgeted for "
                         "8 or for 6 blocks per SM)")
    ap.add_argument("--drift-steps", type=int, default=None,
                    help="untimed steps of the total-energy drift run (default: the 4M Plummer configuration's 100; 0 skips)")
    ap.add_argument("--acc-p", type=int, default=10, help="expansion order of the accurate-mode line")
    ap.add_argument("--acc-steps", type=int, default=3, help="timed steps of each accurate-mode form")
    ap.add_argument("--acc-m2l", default="tf32", choices=["bf16", "tf32"], help="M2L split of the mixed accurate form")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    wdef = {"plummer": (1 << 22, 0.005, 5e-4, 8), "clustered": (1 << 24, 1e-4, 1e-4, 8),
            "uniform": (1 << 20, 1e-3, 1e-4, 6)}[args.workload]
    args.n = wdef[0] if args.n is None else args.n
    args.eps = wdef[1] if args.eps is None else args.eps
    args.dt = wdef[2] if args.dt is None else args.dt
    args.p = wdef[3] if args.p is None else args.p
    if args.drift_steps is None:
        args.drift_steps = 100 if args.workload == "plummer" else 0
    return args


def main():
    args = parse_args()

    if args.impl == "reference":
        run_reference_arm(args)
        return

    ws, rank, local = dist_setup()
    if args.no_tuning_cache:
        os.environ.pop("VIPP_GB_TUNE_FILE", None)
    else:
        os.environ.setdefault("VIPP_GB_TUNE_FILE", SHIPPED_TUNING)
    import torch

    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import vipp_gb300

    base_flags = args.flags
    if args.precision == "mixed" and args.m2l == "bf16":
        args.flags |= vipp_gb300.FLAG_M2L_BF16
    if args.batch_only:
        # the batching form alone (profiling runs); its own line, not the bench contract's
        b = batch_measure(steps=args.batch_steps, warmup=args.warmup, sample=4 if not args.no_error else 0,
                          flags=args.flags & vipp_gb300.FLAG_M2L_BF16, rank=rank, ws=ws, device=local)
        if rank == 0:
            print(json.dumps({"metric": "batching form " + METRIC, "value": b["value"], "unit": UNIT, "batched": b}))
        return
    n = args.n
    t_ic = time.perf_counter()
    x, v, seed, wname = make_workload(args, rank, device=local)
    t_ic = time.perf_counter() - t_ic
    m = 1.0 / n
    sol = vipp_gb300.Solver(p=args.p, s=args.s, eps=args.eps, G=1.0, m=m, precision=args.precision, device=local,
                            flags=args.flags)
    sol.preprocess(x, v)
    if args.p2p_occupancy is not None:
        sol.set_tuning(p2p_occupancy=args.p2p_occupancy)
    tuning_used = sol.tuning()
    for _ in range(args.warmup):
        sol.solve(args.dt)
    sol.sync()
    # total energy before and after the timed steps (untimed; one extra FMM
    # evaluation with potentials each)
    cons0 = sol.conserved() if not args.no_energy else None

    # --- timed region: state resident in HBM -------------------------------------
    # (kernel-class timers off: the step runs as its captured CUDA graph)
    launches0 = sol.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    stream = torch.cuda.ExternalStream(sol.stream_ptr(), device=local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    sol.sync()
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        sol.solve(args.dt)
    ev1.record(stream)
    ev1.synchronize()
    sol.sync()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier(ws)
    elapsed = ev0.elapsed_time(ev1) / 1e3  # device time of exactly --steps steps
    clk = clocks.stop()
    launches = sol.launch_count() - launches0
    st = sol.stats()
    energy = None
    if cons0 is not None:
        cons1 = sol.conserved()
        energy = {"e_before": cons0["total"], "e_after": cons1["total"], "steps": args.steps, "dt": args.dt,
                  "rel_drift": abs(cons1["total"] - cons0["total"]) / abs(cons0["total"]),
                  "potential_from": "FMM far field + FP64 near field of the same method"}
    elapsed = max_over_ranks(elapsed, ws)
    value = n * ws * args.steps / elapsed

    # --- kernel-class breakdown: extra untimed steps with per-class CUDA events --
    class_steps = 2
    sol.enable_timing(True)
    sol.kernel_times()
    for _ in range(class_steps):
        sol.solve(args.dt)
    sol.sync()
    kt = sol.kernel_times()
    sol.enable_timing(False)

    # --- end to end through the C-ABI with pinned host buffers -------------------
    xh = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
    vh = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
    xh.copy_(torch.from_numpy(x))
    vh.copy_(torch.from_numpy(v))
    e2e_steps = max(1, min(args.steps, 3))
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sol.upload_ptr(xh.data_ptr(), vh.data_ptr(), n)
        sol.solve(args.dt)
        sol.download_ptr(xh.data_ptr(), vh.data_ptr())
    e2e_t = max_over_ranks(time.perf_counter() - t0, ws)
    e2e = {"value": n * ws * e2e_steps / e2e_t, "unit": UNIT, "h2d_bytes_per_step": 2 * 24 * n,
           "d2h_bytes_per_step": 2 * 24 * n, "steps": e2e_steps}

    # --- accuracy on a 65,536-particle sample vs the FP64 direct sum (GPU) -------
    acc_info = {}
    if rank == 0 and args.error_sample > 0:
        sol.preprocess(x, v)
        a = sol.accel()
        tg = np.sort(np.random.default_rng(7).choice(n, size=min(args.error_sample, n), replace=False))
        ad = sol.direct_accel(tg)
        e = np.linalg.norm(a[tg] - ad, axis=1) / np.linalg.norm(ad, axis=1)
        acc_info = {"rms_rel_err_vs_fp64_direct": float(math.sqrt(np.mean(e * e))),
                    "max_rel_err_vs_fp64_direct": float(e.max()), "error_sample": int(len(tg))}
    sol.close()

    # --- plain FP64 form of the same method --------------------------------------
    plain = None
    if rank == 0 and not args.no_plain and args.precision == "mixed":
        plain_steps = 2
        with vipp_gb300.Solver(p=args.p, s=args.s, eps=args.eps, m=m, precision="fp64", device=local) as sp:
            sp.preprocess(x, v)
            sp.solve(args.dt)  # captures the step graph
            tp = timed_steps(sp, plain_steps, args.dt, local) / plain_steps
            sp.preprocess(x, v)
            ap64 = sp.accel()
            e = np.linalg.norm(ap64[tg] - ad, axis=1) / np.linalg.norm(ad, axis=1) if acc_info else None
        plain = {"value": n / tp, "unit": UNIT, "steps": plain_steps, "ms_per_step": 1e3 * tp,
                 "timing": f"CUDA events around {plain_steps} steps on the solver's stream",
                 "rms_rel_err_vs_fp64_direct": float(math.sqrt(np.mean(e * e))) if e is not None else None,
                 "max_rel_err_vs_fp64_direct": float(e.max()) if e is not None else None,
                 "mixed_over_plain": value / ws / (n / tp)}

    # --- roofline of the dominant kernel class ---------------------------------
    peaks, src = measured_peaks()
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    props = torch.cuda.get_device_properties(local)
    nsm = props.multi_processor_count
    fp32_peak = 2 * FP32_LANES_PER_SM * nsm * sm_mhz * 1e6 / 1e12  # TFLOP/s
    per = {}
    K = (args.p + 1) ** 2
    if kt["p2p"][1]:
        t = kt["p2p"][0] / kt["p2p"][1] / 1e3
        ach = 20.0 * st["p2p_pairs"] / t / 1e12
        per["p2p"] = {"bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                      "ms_per_launch": 1e3 * t, "launches": kt["p2p"][1]}
    if kt["m2l"][1]:
        t = kt["m2l"][0] / kt["m2l"][1] / 1e3
        ach = 2.0 * K * K * st["m2l_pairs"] / t / 1e12  # algorithmic: one K x K operator per pair
        tensor = args.precision == "mixed" and args.p >= 2 and not (args.flags & vipp_gb300.FLAG_M2L_CUDA_CORES)
        if tensor and args.flags & vipp_gb300.FLAG_M2L_BF16:
            # BF16 hi/lo split: bound = the measured bf16 GEMM rate. Executed work:
            # per tile and slot, K steps of 16 over the [hi | lo] row (2K), N = 2N'
            # where a step reaches hi inputs, else N'.
            nt = max(st["ncells"] - 9, 0)
            tiles = 8 * math.ceil(nt / 8 / 128)
            N = (K + 15) // 16 * 16
            cols = sum(2 * N if 16 * j < K else N for j in range(math.ceil(2 * K / 16)))
            exe = tiles * 189 * 2.0 * 128 * 16 * cols / t / 1e12
            pk = peaks["bf16_tflops"]
            per["m2l"] = {"bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                          "frac": ach / pk, "executed_tflops": exe, "executed_frac": exe / pk,
                          "ms_per_launch": 1e3 * t, "launches": kt["m2l"][1], "split": "bf16 hi/lo",
                          "peak_source": f"{src} bf16_tflops"}
        elif tensor:
            # TF32 tcgen05 MMAs run at half the bf16 rate (same cycles per MMA, half
            # the K), so the bound is half the measured bf16 GEMM rate. Executed
            # tensor work: 128-row tiles of same-octant targets x 189 slots, K and
            # N padded (N to 16, K to 8 per MMA), three hi/lo products.
            tf32_peak = peaks["bf16_tflops"] / 2
            nt = max(st["ncells"] - 9, 0)
            tiles = 8 * math.ceil(nt / 8 / 128)
            N = (K + 15) // 16 * 16
            ksteps = sum(min(4, math.ceil((K - 32 * kc) / 8)) for kc in range(math.ceil(K / 32)))
            exe = tiles * 189 * ksteps * 3 * 2.0 * 128 * N * 8 / t / 1e12
            per["m2l"] = {"bound": "tensor", "achieved": ach, "peak": tf32_peak, "unit": "TFLOP/s",
                          "frac": ach / tf32_peak, "executed_tflops": exe, "executed_frac": exe / tf32_peak,
                          "ms_per_launch": 1e3 * t, "launches": kt["m2l"][1], "split": "3 x tf32",
                          "peak_source": f"{src} bf16_tflops / 2 (TF32 MMA rate)"}
        else:
            per["m2l"] = {"bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                          "ms_per_launch": 1e3 * t, "launches": kt["m2l"][1]}
    if kt["tree"][1]:
        t = kt["tree"][0] / kt["tree"][1] / 1e3
        ncell = st["ncells"]
        ach = (60.0 * n + 64.0 * ncell) / t / 1e9
        per["tree"] = {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                       "frac": ach / peaks["hbm_gbs"], "ms_per_launch": 1e3 * t, "launches": kt["tree"][1]}
    dom = max(per, key=lambda k: per[k]["ms_per_launch"] * per[k]["launches"]) if per else None
    roof = dict(per[dom]) if dom else {}
    if dom:
        # DRAM bytes (read + write) per launch from one ncu capture of this exact
        # default workload; other workloads have no capture, so null
        default_cfg = (args.workload == "plummer" and n == 1 << 22 and args.p == 8 and args.s == 64 and args.eps == 0.005
                       and args.precision == "mixed" and args.flags & ~vipp_gb300.FLAG_M2L_BF16 == 0)
        bf = bool(args.flags & vipp_gb300.FLAG_M2L_BF16)
        traffic = {"p2p": 301173760 + 40833536, "m2l": (M2L_BF16_TRAFFIC if bf else 195950592 + 21233664)} if default_cfg else {}
        for k in per:
            per[k]["traffic"] = traffic.get(k)
        roof.update({"kernel": dom, "traffic": traffic.get(dom), "traffic_unit": "B per launch"})
        roof.setdefault("peak_source", f"{src}: FP32 = 2 x 128 lanes x {nsm} SMs x sm_max_mhz {sm_mhz:.0f}"
                        if roof["bound"] == "fp32" else f"{src} hbm_gbs")

    batched = None
    if not args.no_batch:  # every rank takes its run of the batch's systems
        batched = batch_measure(steps=args.batch_steps, flags=args.flags & vipp_gb300.FLAG_M2L_BF16, rank=rank, ws=ws,
                                device=local)
        batched["m2l_split"] = "bf16 hi/lo" if args.flags & vipp_gb300.FLAG_M2L_BF16 else "3 x tf32"
        if ws == 1 and not args.no_contexts:
            # the same batch as one context per system, for comparison
            ctx_form = batch_measure(steps=10, sample=4, flags=args.flags & vipp_gb300.FLAG_M2L_BF16, form="contexts")
            batched["contexts_form"] = {k: ctx_form[k] for k in ("value", "ms_per_step", "launches_per_step", "steps")}

    # --- the other M2L split on the same workload (value and energy drift) -------
    alt = None
    if rank == 0 and args.precision == "mixed" and not args.no_alt:
        aflags = base_flags if args.flags & vipp_gb300.FLAG_M2L_BF16 else base_flags | vipp_gb300.FLAG_M2L_BF16
        with vipp_gb300.Solver(p=args.p, s=args.s, eps=args.eps, G=1.0, m=m, precision="mixed", device=local,
                               flags=aflags) as sa:
            sa.preprocess(x, v)
            for _ in range(args.warmup):
                sa.solve(args.dt)
            sa.sync()
            ca0 = sa.conserved() if not args.no_energy else None
            sta = torch.cuda.ExternalStream(sa.stream_ptr(), device=local)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            sa.sync()
            e0.record(sta)
            for _ in range(args.steps):
                sa.solve(args.dt)
            e1.record(sta)
            e1.synchronize()
            sa.sync()
            ta = e0.elapsed_time(e1) / 1e3
            drift = None
            if ca0 is not None:
                ca1 = sa.conserved()
                drift = abs(ca1["total"] - ca0["total"]) / abs(ca0["total"])
        alt = {"m2l_split": "bf16 hi/lo" if aflags & vipp_gb300.FLAG_M2L_BF16 else "3 x tf32", "value": n * args.steps / ta,
               "unit": UNIT, "steps": args.steps, "ms_per_step": 1e3 * ta / args.steps, "energy_rel_drift": drift}

    drift = None
    if rank == 0 and args.drift_steps > 0 and args.precision == "mixed":
        # total-energy drift over the configuration's full run (untimed)
        with vipp_gb300.Solver(p=args.p, s=args.s, eps=args.eps, G=1.0, m=m, precision="mixed", device=local,
                               flags=args.flags) as sd:
            sd.preprocess(x, v)
            c0 = sd.conserved()
            t0 = time.perf_counter()
            for _ in range(args.drift_steps):
                sd.solve(args.dt)
            sd.sync()
            tdr = time.perf_counter() - t0
            c1 = sd.conserved()
        drift = {"steps": args.drift_steps, "dt": args.dt, "e_before": c0["total"], "e_after": c1["total"],
                 "rel_drift": abs(c1["total"] - c0["total"]) / abs(c0["total"]), "wall_s": tdr,
                 "m2l_split": "bf16 hi/lo" if args.flags & vipp_gb300.FLAG_M2L_BF16 else "3 x tf32"}

    tuned = None
    if rank == 0 and args.tune:
        # the autotuner on this workload, then the tuned and the default
        # settings timed alike (CUDA events over --steps steps each)
        from vipp_gb300 import autotune
        r = autotune.tune(x, v, p=args.p, s=args.s, eps=args.eps, m=m, precision=args.precision, flags=args.flags,
                          dt=args.dt, steps=2, device=local)
        res = {}
        for label, tset in (("default", vipp_gb300.TUNING_DEFAULT), ("tuned", r["tuning"])):
            with vipp_gb300.Solver(p=args.p, s=args.s, eps=args.eps, G=1.0, m=m, precision=args.precision,
                                   device=local, flags=args.flags) as st_:
                st_.set_tuning(**tset)
                st_.preprocess(x, v)
                st_.solve(args.dt)
                res[label] = n * args.steps / timed_steps(st_, args.steps, args.dt, local)
        tuned = {"tuning": r["tuning"], "bucket": r["key"], "trials": r["trials"], "default_value": res["default"],
                 "tuned_value": res["tuned"], "unit": UNIT, "speedup": res["tuned"] / res["default"]}
        if args.tune_out:
            entries = autotune.read_cache(args.tune_out) if os.path.exists(args.tune_out) else []
            autotune.write_cache(args.tune_out, entries + [(r["key"], r["tuning"])])

    accurate = None
    if rank == 0 and not args.no_accurate and args.precision == "mixed" and acc_info:
        accurate = accurate_measure(x, v, args, local, tg, ad)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(x, args.s, args.p, args.eps)

    kt_ms = {k: round(v[0] / class_steps, 4) for k, v in kt.items()}
    m2l_split = (None if args.precision != "mixed" else "cuda cores fp32" if args.flags & vipp_gb300.FLAG_M2L_CUDA_CORES
                 else "bf16 hi/lo" if args.flags & vipp_gb300.FLAG_M2L_BF16 else "3 x tf32")
    cfg = {"workload": f"{wname} p={args.p} s={args.s} eps={args.eps} {args.precision}", "N": n, "p": args.p,
           "s": args.s, "eps": args.eps, "dt": args.dt, "precision": args.precision, "m2l_split": m2l_split, "seed": seed,
           "l2": f"inputs larger than L2 (state {48 * n / 1e6:.0f} MB, per-step working set > 1 GB)",
           "tree": {k: st[k] for k in ("ncells", "nleaves", "depth", "m2l_pairs", "p2p_pairs", "p2p_ranges")},
           "initial_conditions_s": round(t_ic, 3),
           "tuning_cache": os.environ.get("VIPP_GB_TUNE_FILE"), "tuning": tuning_used,
           "kernel_ms_per_step": kt_ms, **acc_info, "energy": energy, "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed / args.steps, "wall_ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": cfg, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk, "roofline": roof,
            "roofline_kernels": per, "plain_fp64": plain, "accurate": accurate, "energy_drift_run": drift, "autotune": tuned,
            "batched": batched, "m2l_other_split": alt,
            "cpu_baseline": cpu}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
