"""Parity of the CUDA path (through the C-ABI) with the reference and the oracle.

Tolerances (written here, per quantity):
  * tree, cell boxes, member lists, M2L / P2P / colleague lists: bit-exact
    (compared as (level, path) sequences, see treecmp.py);
  * FP64 accelerations: max per-particle relative difference <= 1e-10 from
    the reference's FMM (the special-function evaluation order differs);
  * mixed precision (FP32 P2P / expansions): RMS relative difference <= 2e-6
    and max <= 1e-4 from the reference's FMM; with the BF16 hi/lo split M2L
    (GB_FLAG_M2L_BF16) RMS <= 2e-5 and max <= 1e-4;
  * FP64 RK4 step: positions to 1e-14 and velocities to 1e-11 of their scale.
"""
import math

import numpy as np
import pytest

import oracle as O
from treecmp import canon_gpu, canon_ref, diff_trees, load_case, rel_err

pytestmark = pytest.mark.gpu

CASES = ["plummer2000_s8_p4", "plummer3000_s4_p6", "uniform1500_s16_p3", "cluster1200_s6_p5", "octree3", "octree4",
         "root_leaf28_s10", "split29_s10", "midplane27_s1"]

FP64_MAX_REL = 1e-10
MIXED_RMS_REL = 2e-6
MIXED_MAX_REL = 1e-4
MIXED_BF16_RMS_REL = 2e-5
MIXED_BF16_MAX_REL = 1e-4


def solver(d, precision="fp64"):
    import vipp_gb300
    s = vipp_gb300.Solver(p=d["p"], s=d["s"], eps=d["eps"], G=d["G"], m=d["m"], precision=precision)
    s.preprocess(d["x"], d["v"])
    return s


@pytest.mark.parametrize("name", CASES)
def test_tree_and_lists_bit_exact(name):
    d = load_case(name)
    with solver(d) as s:
        s.accel()
        got = canon_gpu(s.tree_dump())
    assert diff_trees(got, canon_ref(d)) == []


@pytest.mark.parametrize("name", CASES)
def test_fp64_accel_matches_reference(name):
    d = load_case(name)
    with solver(d) as s:
        a = s.accel()
    assert np.max(rel_err(a, d["acc"])) <= FP64_MAX_REL


@pytest.mark.parametrize("name", CASES)
def test_mixed_accel_matches_reference(name):
    d = load_case(name)
    with solver(d, "mixed") as s:
        a = s.accel()
    e = rel_err(a, d["acc"])
    assert math.sqrt(np.mean(e ** 2)) <= MIXED_RMS_REL
    assert np.max(e) <= MIXED_MAX_REL


@pytest.mark.parametrize("name", CASES)
def test_fp64_rk4_step_matches_reference(name):
    d = load_case(name)
    with solver(d) as s:
        s.solve(d["dt"])
        x1, v1 = s.postprocess()
    assert np.max(np.abs(x1 - d["x1"])) <= 1e-14 * max(1.0, np.max(np.abs(d["x"])))
    assert np.max(np.abs(v1 - d["v1"])) <= 1e-11 * max(1e-3, np.max(np.abs(d["v1"])))


@pytest.fixture(scope="module")
def plummer16k():
    """The reference's CPU-runnable case: Problem<double>{16384, s=32, eps=0.01, p=4, seed=0}."""
    x, v = O.plummer_reference(16384, 0.01, 0)
    return x, v


def test_plummer16k_tree_and_accel_vs_oracle(plummer16k):
    import vipp_gb300
    x, v = plummer16k
    n = x.shape[0]
    orc = O.oracle()
    t = orc.tree(x, 32)
    ref_a = orc.accel(x, 32, 1.0, 1.0 / n, 0.01, 4)
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n) as s:
        s.preprocess(x, v)
        a = s.accel()
        assert diff_trees(canon_gpu(s.tree_dump()), canon_ref(t)) == []
        st = s.stats()
    assert np.max(rel_err(a, ref_a)) <= FP64_MAX_REL
    assert st["ncells"] == len(t["parent"]) and st["depth"] == int(t["level"].max())
    assert st["m2l_pairs"] == sum(len(t["m2l"][c]) for c in range(9, len(t["parent"])))
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n, precision="mixed") as s:
        s.preprocess(x, v)
        am = s.accel()
    e = rel_err(am, ref_a)
    assert math.sqrt(np.mean(e ** 2)) <= MIXED_RMS_REL and np.max(e) <= MIXED_MAX_REL


def test_plummer1m_tree_bit_exact_vs_oracle():
    """A million-particle Plummer sphere (reference generator, seed 1, s = 64):
    256 radix tiles per key pass and a 7-8 level tree; the tree, lists and cell
    numbering equal the oracle's, on the first evaluation and on a later one
    (after the sorted key levels have been fitted to the tree)."""
    import vipp_gb300
    x, v = O.plummer_reference(1 << 20, 0.01, 1)
    n = x.shape[0]
    ref = canon_ref(O.oracle().tree(x, 64))
    with vipp_gb300.Solver(p=4, s=64, eps=0.01, m=1.0 / n, precision="mixed") as s:
        s.preprocess(x, v)
        s.accel()
        assert diff_trees(canon_gpu(s.tree_dump()), ref) == []
        r1 = s.stats()["retries"]
        s.accel()
        assert diff_trees(canon_gpu(s.tree_dump()), ref) == []
        assert s.stats()["retries"] == r1  # the fitted levels need no repeat


def test_plummer16k_rk4_trajectory_vs_oracle(plummer16k):
    import vipp_gb300
    x, v = plummer16k
    x, v = x[:4096].copy(), v[:4096].copy()
    n = x.shape[0]
    dt = 1e-3
    xo, vo = O.oracle().rk4(x, v, 32, 1.0, 1.0 / n, 0.01, dt, 4, 3)
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n) as s:
        s.preprocess(x, v)
        for _ in range(3):
            s.solve(dt)
        xg, vg = s.postprocess()
    assert np.max(np.abs(xg - xo)) <= 1e-13 * np.max(np.abs(x))
    assert np.max(np.abs(vg - vo)) <= 1e-10 * np.max(np.abs(v))


def test_direct_sum_kernel_vs_oracle(plummer16k):
    import vipp_gb300
    x, v = plummer16k
    x = x[:3000]
    targets = np.arange(0, 3000, 7)
    ref = O.direct_accel(x, 1.0, 1.0 / 3000, 0.01, targets)
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / 3000) as s:
        s.preprocess(x, np.zeros_like(x))
        a = s.direct_accel(targets)
        a_all = s.direct_accel()
    assert np.max(rel_err(a, ref)) <= 1e-13
    assert np.max(rel_err(a_all[targets], ref)) <= 1e-13


@pytest.mark.parametrize("name", CASES)
def test_mixed_m2l_bf16_split_matches_reference(name):
    """The tensor-core M2L with the BF16 hi/lo split (GB_FLAG_M2L_BF16, ~2^-17
    per product) stays within MIXED_BF16_RMS_REL / MIXED_BF16_MAX_REL of the
    reference's FMM, and the tree it runs on is the same."""
    import vipp_gb300
    d = load_case(name)
    with vipp_gb300.Solver(p=d["p"], s=d["s"], eps=d["eps"], G=d["G"], m=d["m"], precision="mixed",
                           flags=vipp_gb300.FLAG_M2L_BF16) as s:
        s.preprocess(d["x"], d["v"])
        a = s.accel()
        assert diff_trees(canon_gpu(s.tree_dump()), canon_ref(d)) == []
    e = rel_err(a, d["acc"])
    assert math.sqrt(np.mean(e ** 2)) <= MIXED_BF16_RMS_REL and np.max(e) <= MIXED_BF16_MAX_REL


@pytest.mark.parametrize("name", ["plummer3000_s4_p6", "cluster1200_s6_p5", "plummer2000_s8_p4"])
def test_mixed_m2l_tensor_and_cuda_cores_agree(name):
    """The tensor-core M2L (default) and the FP32 CUDA-core M2L both match the reference."""
    import vipp_gb300
    d = load_case(name)
    res = {}
    for label, flags in (("tensor", 0), ("cuda", vipp_gb300.FLAG_M2L_CUDA_CORES)):
        with vipp_gb300.Solver(p=d["p"], s=d["s"], eps=d["eps"], G=d["G"], m=d["m"], precision="mixed", flags=flags) as s:
            s.preprocess(d["x"], d["v"])
            res[label] = s.accel()
        e = rel_err(res[label], d["acc"])
        assert math.sqrt(np.mean(e ** 2)) <= MIXED_RMS_REL and np.max(e) <= MIXED_MAX_REL
    assert np.max(rel_err(res["tensor"], res["cuda"])) <= 2 * MIXED_MAX_REL


@pytest.mark.parametrize("p", [2, 3, 7, 8, 9, 10])
def test_mixed_tensor_m2l_every_order(plummer16k, p):
    """The tensor-core M2L over the expansion orders whose drains differ: the
    running sums in TMEM after both accumulators (p <= 7), in the gaps behind
    them (p = 8), or in registers (p = 9, 10, no free columns). p = 8 against
    the reference itself is in test_gpu_headline.py.
    Mixed against FP64 on the same tree: RMS <= MIXED_RMS_REL, max <= MIXED_MAX_REL."""
    import vipp_gb300
    x, v = plummer16k
    x, v = x[:8192].copy(), v[:8192].copy()
    n = x.shape[0]
    out = {}
    for prec in ("fp64", "mixed"):
        with vipp_gb300.Solver(p=p, s=32, eps=0.01, m=1.0 / n, precision=prec) as s:
            s.preprocess(x, v)
            out[prec] = s.accel()
    e = rel_err(out["mixed"], out["fp64"])
    assert math.sqrt(np.mean(e ** 2)) <= MIXED_RMS_REL and np.max(e) <= MIXED_MAX_REL


def test_results_are_deterministic():
    import vipp_gb300
    d = load_case("cluster1200_s6_p5")
    for prec in ("fp64", "mixed"):
        with vipp_gb300.Solver(p=5, s=6, eps=1e-3, m=d["m"], precision=prec) as s:
            s.preprocess(d["x"], d["v"])
            a1 = s.accel()
            a2 = s.accel()
        assert np.array_equal(a1, a2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_near_field_overflow_is_repeated_cleanly(precision):
    """The first evaluation of a fresh context runs on guessed buffer sizes.
    Plummer 100k (reference generator, seed 0) with s = 256 splits the long
    near-field lists of its leaves into 12,639 partial-sum slots (counted on
    the oracle's tree), three times the initial 4096, so that evaluation
    overflows, queues no P2P work, grows the buffers and is repeated. The
    repeat must equal an evaluation that fits."""
    import vipp_gb300
    x, v = O.plummer_reference(100_000, 0.01, 0)
    with vipp_gb300.Solver(p=4, s=256, eps=0.01, m=1.0 / len(x), precision=precision) as s:
        s.preprocess(x, v)
        a1 = s.accel()
        r1 = s.stats()["retries"]
        a2 = s.accel()
        r2 = s.stats()["retries"]
    assert r1 >= 1 and r2 == r1
    assert np.array_equal(a1, a2)


def test_uniform_cube_mixed_vs_fp64_at_scale():
    """Size-independent property at 262,144 particles: the mixed pipeline agrees
    with the FP64 pipeline (same lists) and the tree is consistent."""
    import vipp_gb300
    rng = np.random.default_rng(5)
    n = 1 << 18
    x = rng.random((n, 3))
    res = {}
    for prec in ("fp64", "mixed"):
        with vipp_gb300.Solver(p=6, s=64, eps=1e-3, m=1.0 / n, precision=prec) as s:
            s.preprocess(x, np.zeros_like(x))
            res[prec] = s.accel()
            if prec == "fp64":
                d = s.tree_dump()
                st = s.stats()
    e = rel_err(res["mixed"], res["fp64"])
    assert math.sqrt(np.mean(e ** 2)) <= MIXED_RMS_REL
    leaf = d["first_child"] < 0
    sizes = d["pt_end"] - d["pt_begin"]
    T = math.floor(math.sqrt(8) * 64)
    assert np.all(sizes[leaf] <= T) and np.all(sizes[~leaf] > T)
    assert np.array_equal(np.sort(d["order"]), np.arange(n))
    assert st["nleaves"] == int(leaf.sum()) and st["p2p_pairs"] > 0


@pytest.mark.parametrize("n,s", [(3000, 1200), (20000, 1000)])
def test_large_leaf_capacity_vs_oracle(n, s):
    """Leaf capacity T = floor(sqrt(8) s) in the thousands: a root-only tree
    (n <= T) and a shallow tree whose leaves hold up to T particles, so the
    within-leaf index sort runs on long leaves with fewer warps per block.
    Tree bit-exact, FP64 accelerations within FP64_MAX_REL of the oracle."""
    import vipp_gb300
    x, v = O.plummer_reference(n, 0.01, 3)
    orc = O.oracle()
    ref = orc.accel(x, s, 1.0, 1.0 / n, 0.01, 4)
    with vipp_gb300.Solver(p=4, s=s, eps=0.01, m=1.0 / n) as sol:
        sol.preprocess(x, v)
        a = sol.accel()
        assert diff_trees(canon_gpu(sol.tree_dump()), canon_ref(orc.tree(x, s))) == []
    assert np.max(rel_err(a, ref)) <= FP64_MAX_REL


def test_edge_cases_and_errors():
    import vipp_gb300
    with vipp_gb300.Solver(p=4, s=4, eps=0.01, m=1.0) as s:
        s.preprocess(np.zeros((0, 3)), np.zeros((0, 3)))  # empty system: no-op
        s.solve(1e-3)
        s.preprocess(np.array([[0.5, 0.5, 0.5]]), np.zeros((1, 3)))
        assert np.all(s.accel() == 0)
        x2 = np.array([[0., 0, 0], [10, 0, 0]])
        s.set_config(eps=1e-4)
        s.preprocess(x2, np.zeros((2, 3)))
        a = s.accel()
        assert a[0, 0] == pytest.approx(10 / (100 + 1e-8) ** 1.5, rel=1e-14)
        # more than floor(sqrt(8) s) coincident particles cannot be separated (the
        # reference recurses without end); the library reports it instead
        s.preprocess(np.ones((20, 3)), np.zeros((20, 3)))
        with pytest.raises(vipp_gb300.GB300Error) as ei:
            s.accel()
        assert ei.value.code == vipp_gb300.GB_ERR_DEPTH
        xb = np.random.default_rng(1).random((50, 3))
        xb[7, 1] = np.nan
        s.preprocess(xb, np.zeros_like(xb))
        with pytest.raises(vipp_gb300.GB300Error) as ei:
            s.accel()
        assert ei.value.code == vipp_gb300.GB_ERR_NONFINITE
        # the context stays usable after an error
        s.preprocess(x2, np.zeros((2, 3)))
        assert s.accel()[0, 0] > 0
    with vipp_gb300.Solver(p=4, s=4) as s:
        with pytest.raises(vipp_gb300.GB300Error) as ei:
            s.solve(1e-3)
        assert ei.value.code == vipp_gb300.GB_ERR_STATE


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replayed_steps_equal_direct_launches(plummer16k, precision):
    """RK4 steps replayed from the captured CUDA graph give exactly the
    results of launching every kernel (GB_FLAG_NO_GRAPH), across a change of
    dt (re-capture), a new upload of a different size (re-capture) and new
    data of the same size (replayed without re-capture)."""
    import vipp_gb300
    x, v = plummer16k
    out = []
    for flags in (0, vipp_gb300.FLAG_NO_GRAPH):
        with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / len(x), precision=precision, flags=flags) as s:
            s.preprocess(x, v)
            for dt in (1e-3, 1e-3, 2e-3, 2e-3):
                s.solve(dt)
            a = s.postprocess()
            s.preprocess(x[:5000], v[:5000])
            s.solve(1e-3)
            s.solve(1e-3)
            b = s.postprocess()
            caps = s.stats()["graph_captures"]
            # new data of the same size: the captured graph is replayed as is
            s.preprocess(x[5000:10000], v[5000:10000])
            s.solve(1e-3)
            s.solve(1e-3)
            st = s.stats()
            out.append((a, b, s.postprocess(), s.launch_count(), st, st["graph_captures"] - caps))
    (a0, b0, c0, l0, st0, new0), (a1, b1, c1, l1, st1, new1) = out
    assert st0["graph_steps"] == 8 and st0["direct_steps"] == 0  # the graph path really ran
    assert st1["graph_steps"] == 0 and st1["direct_steps"] == 8
    assert st1["graph_captures"] == 0 and new0 == 0 and st0["graph_captures"] >= 3
    assert np.array_equal(a0[0], a1[0]) and np.array_equal(a0[1], a1[1])
    assert np.array_equal(b0[0], b1[0]) and np.array_equal(b0[1], b1[1])
    assert np.array_equal(c0[0], c1[0]) and np.array_equal(c0[1], c1[1])
    assert l0 == l1
