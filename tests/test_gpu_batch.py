"""Batches of independent systems (gb_batch_*), in both forms: every system of
a batch step must equal the same system stepped alone in its own context, bit
for bit, in both precisions and with each M2L path (tensor cores with either
split, CUDA cores); uneven sizes, an empty and a one-particle system,
per-system masses, and a system whose first step overflows its buffers
(repeated). The forest form (one context, one launch per kernel class over all
systems) is also compared with the contexts form on many systems: positions,
velocities, accelerations, potentials, tree totals and initial conditions."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

FORMS = ("forest", "contexts")


def systems():
    out = []
    for k, n in enumerate([1500, 1, 0, 3000, 2048]):
        x, v = O.plummer_reference(n, 0.01, 10 + k) if n > 1 else (np.full((n, 3), 0.25), np.zeros((n, 3)))
        out.append((x * (0.5 + 0.3 * k), v / np.sqrt(0.5 + 0.3 * k)))
    return out


def form_flags(form):
    import vipp_gb300
    return vipp_gb300.FLAG_BATCH_CONTEXTS if form == "contexts" else 0


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("precision,m2l", [("fp64", ""), ("mixed", "tf32"), ("mixed", "bf16"), ("mixed", "cuda")])
def test_batch_equals_separate_contexts(form, precision, m2l):
    import vipp_gb300
    flags = {"": 0, "tf32": 0, "bf16": vipp_gb300.FLAG_M2L_BF16, "cuda": vipp_gb300.FLAG_M2L_CUDA_CORES}[m2l]
    sy = systems()
    sizes = [len(x) for x, _ in sy]
    masses = [1.0 / max(n, 1) for n in sizes]
    X = np.concatenate([x for x, _ in sy]) if sum(sizes) else np.zeros((0, 3))
    V = np.concatenate([v for _, v in sy])
    with vipp_gb300.Batch(sizes, p=5, s=16, eps=0.01, masses=masses, precision=precision,
                          flags=flags | form_flags(form)) as b:
        assert b.forest == (form == "forest")
        b.upload(X, V)
        for dt in (1e-3, 1e-3, 2e-3):
            b.step(dt)
        xb, vb = b.download()
        a3 = b.system_accel(3)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k, (x, v) in enumerate(sy):
        if len(x) == 0:
            continue
        with vipp_gb300.Solver(p=5, s=16, eps=0.01, m=masses[k], precision=precision, flags=flags) as s:
            s.preprocess(x, v)
            for dt in (1e-3, 1e-3, 2e-3):
                s.solve(dt)
            xs, vs = s.postprocess()
            if k == 3:
                assert np.array_equal(s.accel(), a3)
        assert np.array_equal(xb[off[k]:off[k + 1]], xs) and np.array_equal(vb[off[k]:off[k + 1]], vs)


@pytest.mark.parametrize("form", FORMS)
def test_batch_system_overflow_is_repeated(form):
    import vipp_gb300
    x, v = O.plummer_reference(100_000, 0.01, 0)  # needs 3x the initial partial-sum slots at s = 256
    y, w = O.plummer_reference(4000, 0.01, 1)
    sizes = [len(y), len(x)]
    with vipp_gb300.Batch(sizes, p=4, s=256, eps=0.01, masses=[1 / len(y), 1 / len(x)], precision="mixed",
                          flags=form_flags(form)) as b:
        b.upload(np.concatenate([y, x]), np.concatenate([w, v]))
        b.step(1e-3)
        xb, vb = b.download()
    with vipp_gb300.Solver(p=4, s=256, eps=0.01, m=1 / len(x), precision="mixed") as s:
        s.preprocess(x, v)
        s.solve(1e-3)
        xs, vs = s.postprocess()
    assert np.array_equal(xb[len(y):], xs) and np.array_equal(vb[len(y):], vs)


@pytest.mark.parametrize("precision,flags", [("mixed", 16), ("mixed", 0), ("fp64", 0)])
def test_forest_equals_contexts_many_systems(precision, flags):
    """96 Plummer systems drawn on the device (N log-uniform in [16, 6000],
    radii in [0.5, 2]): the forest and the contexts form give the same initial
    conditions, the same tree totals and, after two steps, the same state,
    accelerations and potentials, bit for bit; conserved quantities agree."""
    import vipp_gb300
    rng = np.random.default_rng(5)
    sizes = np.rint(np.exp(rng.uniform(math.log(16), math.log(6000), 96))).astype(np.int64)
    sizes[7] = 0
    sizes[11] = 1
    masses = 1.0 / np.maximum(sizes, 1)
    res = {}
    for form in FORMS:
        with vipp_gb300.Batch(sizes, p=6, s=32, eps=0.01, masses=masses, precision=precision,
                              flags=flags | form_flags(form)) as b:
            radii = b.init_plummer(seed=9)
            x0, v0 = b.download()
            b.step(1e-3)
            b.step(1e-3)
            x, v = b.download()
            a, phi = b.accel(potential=True)
            res[form] = dict(radii=radii, x0=x0, v0=v0, x=x, v=v, a=a, phi=phi, stats=b.stats(),
                             cons=b.conserved())
    f, c = res["forest"], res["contexts"]
    for k in ("radii", "x0", "v0", "x", "v", "a", "phi"):
        assert np.array_equal(f[k], c[k]), k
    # an empty system's context never evaluates; the forest gives it a root leaf
    empty = int(np.sum(sizes == 0))
    for k in ("n", "ncells", "nleaves", "depth", "m2l_pairs", "p2p_pairs", "p2p_ranges"):
        assert f["stats"][k] == c["stats"][k] + (empty if k in ("ncells", "nleaves") else 0), k
    for cf, cc in zip(f["cons"], c["cons"]):
        for k in ("kinetic", "potential"):
            assert cf[k] == pytest.approx(cc[k], rel=1e-12, abs=1e-300)


def test_forest_launches_do_not_grow_with_systems():
    """One forest step queues the same kernels whatever the number of systems
    (the step graph's launch count; contexts: one graph per system), up to one
    more radix pass per force evaluation for the wider system index."""
    import vipp_gb300
    counts = {}
    for nsys in (8, 64):
        sizes = np.full(nsys, 2000)
        with vipp_gb300.Batch(sizes, p=4, s=32, eps=0.01, masses=1.0 / sizes, precision="mixed") as b:
            b.init_plummer(seed=1)
            b.step(1e-3)
            b.step(1e-3)
            l0 = b.launch_count()
            b.step(1e-3)
            counts[nsys] = b.launch_count() - l0
    assert counts[8] <= counts[64] <= counts[8] + 16 and counts[64] < 300, counts


def test_forest_depth_beyond_its_sort_word_is_reported():
    """1024 systems leave 18 key levels beside the system index: a system
    whose tree needs more fails the step with GB_ERR_DEPTH (the contexts form
    runs it)."""
    import vipp_gb300
    sizes = np.zeros(1024, dtype=np.int64)
    # six particles 4e-7 apart in a unit box: the tree reaches level 20 (the oracle's tree of it)
    deep = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]] + [[0.3 + 4e-7 * i, 0.3, 0.3] for i in range(6)])
    sizes[5] = len(deep)
    with vipp_gb300.Batch(sizes, p=3, s=1, eps=0.01, masses=np.ones(1024), precision="mixed") as b:
        b.upload(deep, np.zeros_like(deep))
        with pytest.raises(vipp_gb300.GB300Error) as e:
            b.step(1e-3)
        assert e.value.code == vipp_gb300.GB_ERR_DEPTH
    with vipp_gb300.Batch(sizes, p=3, s=1, eps=0.01, masses=np.ones(1024), precision="mixed",
                          flags=vipp_gb300.FLAG_BATCH_CONTEXTS) as b:
        b.upload(deep, np.zeros_like(deep))
        b.step(1e-3)


def test_accurate_mode_batch_runs_as_contexts():
    """The accurate mode's batches take the contexts form (the forest builds
    the reference mode's tree only), with the same per-system results."""
    import vipp_gb300
    sy = systems()[:2]
    sizes = [len(x) for x, _ in sy]
    masses = [1.0 / n for n in sizes]
    with vipp_gb300.Batch(sizes, p=6, s=16, eps=0.01, masses=masses, precision="mixed", mode="accurate") as b:
        assert not b.forest
        b.upload(np.concatenate([x for x, _ in sy]), np.concatenate([v for _, v in sy]))
        a = b.accel()
    with vipp_gb300.Solver(p=6, s=16, eps=0.01, m=masses[1], precision="mixed", mode="accurate") as s:
        s.preprocess(*sy[1])
        assert np.array_equal(s.accel(), a[sizes[0]:])


def test_forest_equals_contexts_on_the_benchmark_batch():
    """bench.py's batching form (512 Plummer systems, N log-uniform in
    [1024, 65536], 7.5 M particles, BF16 split): one batch step of the forest
    and of one context per system give the same positions and velocities, bit
    for bit."""
    import vipp_gb300
    rng = np.random.default_rng(3)
    sizes = np.rint(np.exp(rng.uniform(math.log(1024), math.log(65536), 512))).astype(np.int64)
    out = {}
    for form in FORMS:
        with vipp_gb300.Batch(sizes, p=6, s=32, eps=0.01, masses=1.0 / sizes, precision="mixed",
                              flags=vipp_gb300.FLAG_M2L_BF16 | form_flags(form)) as b:
            b.init_plummer(seed=3)
            b.step(1e-3)
            out[form] = b.download()
    assert np.array_equal(out["forest"][0], out["contexts"][0])
    assert np.array_equal(out["forest"][1], out["contexts"][1])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_step_repeated_after_overflow_equals_step_without(precision):
    """A step whose first attempt overflows a buffer is grown and run again
    from the step's start: the same result as a step that needed no repeat
    (the RK4 sums start over at stage 0)."""
    import vipp_gb300
    x, v = O.plummer_reference(100_000, 0.01, 0)  # needs 3x the initial partial-sum slots at s = 256
    n = len(x)
    with vipp_gb300.Solver(p=4, s=256, eps=0.01, m=1 / n, precision=precision) as a:
        a.preprocess(x, v)
        a.solve(1e-3)
        xa, va = a.postprocess()
        ra = a.stats()["retries"]
    with vipp_gb300.Solver(p=4, s=256, eps=0.01, m=1 / n, precision=precision) as b:
        b.preprocess(x, v)
        b.accel()  # grows the buffers outside the step
        rb0 = b.stats()["retries"]
        b.solve(1e-3)
        xb, vb = b.postprocess()
        rb = b.stats()["retries"] - rb0
    assert ra >= 1 and rb == 0
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


@pytest.mark.parametrize("sizes", [[3000], [5, 10, 0, 3, 90], [91, 1, 2000]])
def test_forest_edge_batches(sizes):
    """Forests of one system, of systems that are single leaves (no far
    field at all: every root holds at most floor(sqrt(8) s) particles), and
    of a system just over one leaf beside tiny ones: each system equals its own
    context after two steps, and its accelerations match."""
    import vipp_gb300
    sy = []
    for k, n in enumerate(sizes):
        x, v = O.plummer_reference(n, 0.01, 40 + k) if n > 1 else (np.full((n, 3), 0.5), np.zeros((n, 3)))
        sy.append((x, v))
    masses = [1.0 / max(n, 1) for n in sizes]
    X = np.concatenate([x for x, _ in sy])
    V = np.concatenate([v for _, v in sy])
    with vipp_gb300.Batch(sizes, p=5, s=32, eps=0.01, masses=masses, precision="mixed") as b:
        assert b.forest
        b.upload(X, V)
        b.step(1e-3)
        b.step(1e-3)
        xb, vb = b.download()
        ab = b.accel()
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k, (x, v) in enumerate(sy):
        if len(x) == 0:
            continue
        with vipp_gb300.Solver(p=5, s=32, eps=0.01, m=masses[k], precision="mixed") as s:
            s.preprocess(x, v)
            s.solve(1e-3)
            s.solve(1e-3)
            xs, vs = s.postprocess()
            a = s.accel()
        sl = slice(off[k], off[k + 1])
        assert np.array_equal(xb[sl], xs) and np.array_equal(vb[sl], vs) and np.array_equal(ab[sl], a)
