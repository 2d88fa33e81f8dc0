"""Parity at the benchmark's own orders and leaf capacity, and over the
reference's CPU-runnable case run to its end, through the C-ABI.

Fixtures (tests/golden/make_golden.py, from the reference's headers compiled
unmodified):
  * tree_plummer16384_s64_p8: Problem::initialize (problem.hpp:188-211),
    N = 16,384, eps = 0.005, p = 8, s = 64 (the 4M Plummer configuration's
    order, leaf capacity and softening; 529 cells, depth 7);
  * tree_uniform16384_s64_p6: unit cube, eps = 1e-3, p = 6, s = 64 (the
    plain-at-scale configuration's shape; depth 3);
  * traj_plummer16384_s32_p4: N = 16,384, s = 32, eps = 0.01, p = 4, ten RK4
    steps of dt = 1e-3 (solver_ref.hpp:36-104).

Tolerances (per quantity):
  * tree, boxes, member lists, M2L / P2P / colleague lists: bit-exact;
  * FP64 accelerations: max per-particle relative difference <= 1e-10;
  * mixed, tensor-core M2L with the 3 x TF32 split (the library default):
    RMS <= 2e-6, max <= 1e-4;
  * mixed, BF16 hi/lo split (GB_FLAG_M2L_BF16, the benchmark's form):
    RMS <= 2e-5, max <= 1e-4;
  * ten-step trajectory, FP64: positions within 1e-13 and velocities within
    1e-11 absolute (the state's scale is ~1);
  * ten-step trajectory, mixed: per particle, the velocity difference divided
    by the reference's velocity change over the run (the effective relative
    error of the mean acceleration) has RMS <= the acceleration tolerance of
    the split and max <= 1e-3; positions within 1e-8 absolute.
"""
import math

import numpy as np
import pytest

from treecmp import GOLDEN, canon_gpu, canon_ref, checksum, diff_trees, load_case, regenerate, rel_err

pytestmark = pytest.mark.gpu

BIG = ["plummer16384_s64_p8", "uniform16384_s64_p6"]
FP64_MAX_REL = 1e-10
TF32_RMS, BF16_RMS, MIXED_MAX = 2e-6, 2e-5, 1e-4


def run(d, precision="fp64", flags=0):
    import vipp_gb300
    with vipp_gb300.Solver(p=d["p"], s=d["s"], eps=d["eps"], G=d["G"], m=d["m"], precision=precision,
                           flags=flags) as s:
        s.preprocess(d["x"], d["v"])
        a = s.accel()
        tree = canon_gpu(s.tree_dump())
        st = s.stats()
    return a, tree, st


@pytest.fixture(scope="module", params=BIG)
def case(request):
    return request.param, load_case(request.param)


def test_tree_bit_exact(case):
    name, d = case
    _, tree, st = run(d)
    assert diff_trees(tree, canon_ref(d)) == []
    assert st["ncells"] == len(d["parent"]) and st["depth"] == int(d["level"].max())


def test_fp64(case):
    name, d = case
    a, _, _ = run(d)
    assert np.max(rel_err(a, d["acc"])) <= FP64_MAX_REL


def test_mixed_tf32_split(case):
    name, d = case
    a, tree, _ = run(d, "mixed")
    e = rel_err(a, d["acc"])
    assert math.sqrt(np.mean(e ** 2)) <= TF32_RMS and np.max(e) <= MIXED_MAX
    assert diff_trees(tree, canon_ref(d)) == []


def test_mixed_bf16_split(case):
    import vipp_gb300
    name, d = case
    a, tree, _ = run(d, "mixed", vipp_gb300.FLAG_M2L_BF16)
    e = rel_err(a, d["acc"])
    assert math.sqrt(np.mean(e ** 2)) <= BF16_RMS and np.max(e) <= MIXED_MAX
    assert diff_trees(tree, canon_ref(d)) == []


def test_mixed_cuda_core_m2l(case):
    """The FP32 CUDA-core M2L (GB_FLAG_M2L_CUDA_CORES) at the same orders."""
    import vipp_gb300
    name, d = case
    a, _, _ = run(d, "mixed", vipp_gb300.FLAG_M2L_CUDA_CORES)
    e = rel_err(a, d["acc"])
    assert math.sqrt(np.mean(e ** 2)) <= TF32_RMS and np.max(e) <= MIXED_MAX


@pytest.fixture(scope="module")
def traj():
    z = np.load(f"{GOLDEN}/traj_plummer16384_s32_p4.npz")
    d = {k: z[k] for k in z.files}
    d["x"], d["v"] = regenerate(d["gen"])
    assert np.array_equal(checksum(d["x"]), d["x_sum"]) and np.array_equal(checksum(d["v"]), d["v_sum"])
    return d


def steps(d, precision, flags=0):
    import vipp_gb300
    with vipp_gb300.Solver(p=int(d["p"]), s=int(d["s"]), eps=float(d["eps"]), G=float(d["G"]), m=float(d["m"]),
                           precision=precision, flags=flags) as s:
        s.preprocess(d["x"], d["v"])
        for _ in range(int(d["steps"])):
            s.solve(float(d["dt"]))
        return s.postprocess()


def test_ten_step_trajectory_fp64(traj):
    x, v = steps(traj, "fp64")
    assert np.max(np.abs(x - traj["x10"])) <= 1e-13
    assert np.max(np.abs(v - traj["v10"])) <= 1e-11


@pytest.mark.parametrize("split", ["tf32", "bf16"])
def test_ten_step_trajectory_mixed(traj, split):
    import vipp_gb300
    x, v = steps(traj, "mixed", vipp_gb300.FLAG_M2L_BF16 if split == "bf16" else 0)
    dv = np.linalg.norm(traj["v10"] - traj["v"], axis=1)
    e = np.linalg.norm(v - traj["v10"], axis=1) / dv
    assert math.sqrt(np.mean(e ** 2)) <= (BF16_RMS if split == "bf16" else TF32_RMS)
    assert np.max(e) <= 1e-3
    assert np.max(np.abs(x - traj["x10"])) <= 1e-8
