"""Autotuner of the solver's launch and tree parameters, per size bucket.

The knobs are the gb_tuning fields of include/vipp_gb300.h:

  p2p_blocks       P2P blocks per SM when the near field runs alone
  p2p_blocks_conc  P2P blocks per SM launched beside the far field (the
                   near field's share of the SMs while M2L runs)
  p2p_slice        near-field sources per P2P work item (the near field's
                   work-item size: load balance against per-item overhead)
  m2l_ctas_pct     tensor-core M2L CTAs as a percent of the SMs (its tile
                   schedule: how many persistent CTAs share the 128-target tiles)
  serial           near field after the far field instead of beside it
  p2p_occupancy    mixed P2P kernel build: registers budgeted for 8 or for
                   6 resident blocks per SM
  leaf_s           leaf capacity, in the accurate mode only (the reference
                   mode keeps the reference's s so its trees stay the
                   reference's); candidates are >= the configured s, whose
                   larger near field keeps the accuracy

A bucket is (p, precision, mode, M2L split, floor(log2 n)). ``tune`` measures
one RK4 step per candidate (wall clock around synchronised steps, after one
untimed step that captures the step graph) by coordinate descent from the
defaults: each knob in turn over its candidates, the others held at the best
so far, two sweeps. ``write_cache`` writes the entries in the file format that
gb_tuning_lookup reads (and gb_upload applies when VIPP_GB_TUNE_FILE names
the file).

    python -m vipp_gb300.autotune --workload plummer --n 4194304 --out tune.txt
"""
from __future__ import annotations

import argparse
import math
import os
import time

from . import MODE, PREC, TUNING_DEFAULT, TUNING_FIELDS, FLAG_M2L_BF16, Solver

CANDIDATES = {
    "p2p_blocks": (4, 6, 8),
    "p2p_blocks_conc": (0, 2, 4, 6, 8),
    "p2p_slice": (2048, 4096, 8192, 16384, 32768),
    "m2l_ctas_pct": (50, 75, 100),
    "serial": (0, 1),
    "p2p_occupancy": (8, 6),
}


def bucket_key(n: int, p: int, precision: str, mode: str, flags: int) -> dict:
    return {"p": int(p), "precision": PREC[precision], "mode": MODE[mode],
            "m2l_bf16": 1 if flags & FLAG_M2L_BF16 else 0, "log2n": int(math.floor(math.log2(n)))}


def cache_line(key: dict, tuning: dict, comment: str = "") -> str:
    toks = [f"{k}={int(key[k])}" for k in ("p", "precision", "mode", "m2l_bf16", "log2n")]
    toks += [f"{k}={int(tuning[k])}" for k in TUNING_FIELDS]
    return " ".join(toks) + (f"  # {comment}" if comment else "")


def write_cache(path: str, entries) -> None:
    """entries: iterable of (key, tuning[, comment]); later entries of the same
    bucket win when the file is read."""
    with open(path, "w") as f:
        f.write("# vipp-gb300 tuning cache: one entry per line (gb_tuning_lookup)\n")
        for e in entries:
            f.write(cache_line(*e) + "\n")


def read_cache(path: str) -> list:
    out = []
    with open(path) as f:
        for ln in f:
            ln = ln.split("#", 1)[0].strip()
            if not ln:
                continue
            kv = dict(t.split("=", 1) for t in ln.split())
            out.append(({k: int(kv[k]) for k in ("p", "precision", "mode", "m2l_bf16", "log2n")},
                        {k: int(kv.get(k, TUNING_DEFAULT[k])) for k in TUNING_FIELDS}))
    return out


def step_seconds(sol: Solver, dt: float, steps: int) -> float:
    sol.solve(dt)  # captures the step graph for this tuning
    sol.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        sol.solve(dt)
    sol.sync()
    return (time.perf_counter() - t0) / steps


def tune(x, v, *, p: int, s: int, eps: float, m: float, G: float = 1.0, precision: str = "mixed", mode: str = "ref",
         flags: int = 0, dt: float = 1e-4, steps: int = 2, sweeps: int = 2, leaf_s_candidates=None, device: int = 0,
         log=None) -> dict:
    """Best tuning for this workload by coordinate descent; returns
    {"key", "tuning", "default_s", "tuned_s", "trials"} (seconds per step)."""
    cands = dict(CANDIDATES)
    if mode == "accurate":
        cands["leaf_s"] = tuple(leaf_s_candidates or (0, s + s // 4, s + s // 2))
    trials = []
    with Solver(p=p, s=s, eps=eps, G=G, m=m, precision=precision, device=device, flags=flags, mode=mode) as sol:
        sol.preprocess(x, v)
        best = dict(TUNING_DEFAULT)

        def measure(t):
            sol.set_tuning(**t)
            sec = step_seconds(sol, dt, steps)
            trials.append((dict(t), sec))
            if log:
                log(f"  {t} -> {1e3 * sec:.2f} ms/step")
            return sec

        default_s = measure(best)
        best_s = default_s
        for _ in range(sweeps):
            changed = False
            for knob, values in cands.items():
                for val in values:
                    if val == best[knob]:
                        continue
                    t = dict(best)
                    t[knob] = val
                    sec = measure(t)
                    if sec < best_s * 0.995:  # keep a change only when it is clearly faster
                        best, best_s, changed = t, sec, True
            if not changed:
                break
        # the defaults and the winner once more, alternating, against drift of the GPU clock
        d2, b2 = measure(dict(TUNING_DEFAULT)), measure(best)
        if d2 < b2:
            best, b2 = dict(TUNING_DEFAULT), d2
    return {"key": bucket_key(len(x), p, precision, mode, flags), "tuning": best, "default_s": min(default_s, d2),
            "tuned_s": b2, "trials": len(trials)}


def main(argv=None):
    from .workloads import clustered, plummer, uniform

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="plummer", choices=["plummer", "clustered", "uniform"])
    ap.add_argument("--n", type=int, default=1 << 22)
    ap.add_argument("--p", type=int, default=8)
    ap.add_argument("--s", type=int, default=64)
    ap.add_argument("--eps", type=float, default=0.005)
    ap.add_argument("--precision", default="mixed", choices=list(PREC))
    ap.add_argument("--mode", default="ref", choices=list(MODE))
    ap.add_argument("--flags", type=int, default=FLAG_M2L_BF16)
    ap.add_argument("--dt", type=float, default=5e-4)
    ap.add_argument("--out", default="tune.txt")
    a = ap.parse_args(argv)
    if a.workload == "plummer":
        x, v = plummer(a.n, 2)
    elif a.workload == "uniform":
        x, v = uniform(a.n, 1)
    else:
        x, v, _ = clustered(a.n, 4)
    r = tune(x, v, p=a.p, s=a.s, eps=a.eps, m=1.0 / a.n, precision=a.precision, mode=a.mode, flags=a.flags, dt=a.dt,
             log=print)
    entries = read_cache(a.out) if os.path.exists(a.out) else []
    entries.append((r["key"], r["tuning"]))
    write_cache(a.out, entries)
    print(f"default {1e3 * r['default_s']:.2f} ms/step, tuned {1e3 * r['tuned_s']:.2f} ms/step: {r['tuning']}")


if __name__ == "__main__":
    main()
