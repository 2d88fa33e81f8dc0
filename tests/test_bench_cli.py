"""bench.py's command line and its reference arm on the CPU: the default
workload and its sizes, the clustered workload's defaults, the warm-up floor,
and the JSON line of ``--impl reference`` (the oracle on the host cores)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    # imported by the tests, not at collection: bench.py sets
    # CUDA_DEVICE_MAX_CONNECTIONS for its own process
    import bench as b
    return b


def test_default_workload_is_the_4m_plummer_sphere(bench):
    a = bench.parse_args([])
    assert (a.workload, a.n, a.p, a.s, a.eps, a.dt) == ("plummer", 1 << 22, 8, 64, 0.005, 5e-4)
    assert (a.precision, a.m2l, a.impl, a.gpus, a.steps, a.warmup) == ("mixed", "bf16", "gb300", 1, 10, 3)


def test_clustered_defaults_and_explicit_values_win(bench):
    a = bench.parse_args(["--workload", "clustered"])
    assert (a.n, a.eps, a.dt, a.p, a.s) == (1 << 24, 1e-4, 1e-4, 8, 64)
    b = bench.parse_args(["--workload", "clustered", "--n", "4096", "--eps", "0.01", "--dt", "0.001", "--p", "5"])
    assert (b.n, b.eps, b.dt, b.p) == (4096, 0.01, 0.001, 5)
    u = bench.parse_args(["--workload", "uniform"])
    assert (u.n, u.eps, u.dt, u.p, u.s) == (1 << 20, 1e-3, 1e-4, 6, 64)


def test_warmup_floor_applies_to_the_gpu_arm_only(bench):
    assert bench.parse_args(["--warmup", "1"]).warmup == 3
    assert bench.parse_args(["--warmup", "1", "--impl", "reference"]).warmup == 1


def test_workloads_are_seeded_per_replica(bench):
    a = bench.parse_args(["--n", "2048"])
    x0, v0, s0, name = bench.make_workload(a, 0)
    x1, _, s1, _ = bench.make_workload(a, 1)
    assert (s0, s1) == (2, 3) and name == "plummer-2048" and x0.shape == (2048, 3) and v0.shape == (2048, 3)
    assert not np.array_equal(x0, x1)
    c = bench.parse_args(["--workload", "clustered", "--n", "2048"])
    xc, _, sc, namec = bench.make_workload(c, 0)
    assert sc == 4 and namec.startswith("clustered-2048") and xc.shape == (2048, 3)
    u = bench.parse_args(["--workload", "uniform", "--n", "2048"])
    xu, vu, su, nameu = bench.make_workload(u, 0)
    assert su == 1 and nameu.startswith("uniform-2048") and np.all((xu >= 0) & (xu < 1)) and not vu.any()


def test_reference_arm_prints_one_contract_line(bench):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "8192", "--steps", "1"], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["value"] > 0 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["N"] == 8192 and d["config"]["workload"].startswith("plummer-8192")
