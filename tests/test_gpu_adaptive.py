"""The adaptive-depth stress workload on the GPU: 8 equal-mass Plummer clusters
(scale radii uniform in [0.01, 0.1], centres uniform in [0, 1)^3) plus a 5%
uniform background (vipp_gb300.workloads.clustered), eps = 1e-4, s = 64, p = 8.

Tolerances (written here, per quantity):
  * 1,048,576 particles: tree, cell boxes, member lists and M2L / P2P /
    colleague lists bit-exact with the oracle's (compared as (level, path)
    sequences, see treecmp.py), on the first evaluation and after the sorted
    key levels are fitted; the mixed pipeline with the BF16 hi/lo M2L split
    within BF16_RMS_REL (RMS) and BF16_MAX_REL (max) relative difference of
    the FP64 pipeline on the same tree;
  * 16,777,216 particles (the full workload), size-independent properties of
    one evaluation: every leaf holds at most T = floor(sqrt(8) s) particles
    and every internal cell more; children's particle counts add up to their
    parent's; every particle lies inside its leaf's box; the tree order is a
    permutation; the M2L pair count equals the lists' lengths; the FMM
    acceleration is within DIRECT_RMS_REL (RMS) of the FP64 direct sum on a
    2,048-particle sample.
"""
import math

import numpy as np
import pytest

import oracle as O
from treecmp import canon_gpu, canon_ref, diff_trees, rel_err

pytestmark = pytest.mark.gpu

EPS = 1e-4
S = 64
P = 8
BF16_RMS_REL = 2e-5
BF16_MAX_REL = 1e-3
DIRECT_RMS_REL = 5e-3


def _workload(n):
    from vipp_gb300.workloads import clustered
    x, v, _ = clustered(n, 4)
    return x, v


def test_clustered1m_tree_bit_exact_and_bf16_vs_fp64():
    import vipp_gb300
    n = 1 << 20
    x, v = _workload(n)
    ref = canon_ref(O.oracle().tree(x, S))
    acc = {}
    for prec, flags in (("fp64", 0), ("mixed", vipp_gb300.FLAG_M2L_BF16)):
        with vipp_gb300.Solver(p=P, s=S, eps=EPS, m=1.0 / n, precision=prec, flags=flags) as s:
            s.preprocess(x, v)
            acc[prec] = s.accel()
            if prec == "mixed":
                assert diff_trees(canon_gpu(s.tree_dump()), ref) == []
                r1 = s.stats()["retries"]
                a2 = s.accel()  # the sorted key levels are fitted to the tree now
                assert diff_trees(canon_gpu(s.tree_dump()), ref) == []
                assert s.stats()["retries"] == r1
                assert np.array_equal(a2, acc[prec])
    e = rel_err(acc["mixed"], acc["fp64"])
    rms, mx = math.sqrt(np.mean(e * e)), float(np.max(e))
    print(f"clustered 1M: mixed (BF16 M2L) vs FP64 pipeline RMS {rms:.3e} max {mx:.3e}")
    assert rms <= BF16_RMS_REL and mx <= BF16_MAX_REL


def test_clustered16m_tree_properties_and_error_vs_direct():
    import vipp_gb300
    n = 1 << 24
    x, v = _workload(n)
    with vipp_gb300.Solver(p=P, s=S, eps=EPS, m=1.0 / n, precision="mixed", flags=vipp_gb300.FLAG_M2L_BF16) as s:
        s.preprocess(x, v)
        a = s.accel()
        st = s.stats()
        d = s.tree_dump()
        tg = np.sort(np.random.default_rng(11).choice(n, size=2048, replace=False))
        ad = s.direct_accel(tg)
    T = math.floor(math.sqrt(8) * S)
    C = len(d["level"])
    leaf = d["first_child"] < 0
    size = d["pt_end"] - d["pt_begin"]
    print(f"clustered 16M: {C} cells, {int(leaf.sum())} leaves, depth {st['depth']}, "
          f"{st['m2l_pairs']} M2L pairs, {st['p2p_pairs']} P2P pairs")
    assert st["ncells"] == C and st["nleaves"] == int(leaf.sum()) and st["depth"] == int(d["level"].max())
    assert np.all(size[leaf] <= T) and np.all(size[~leaf] > T) and size[0] == n
    child_sum = np.bincount(d["parent"][1:], weights=size[1:], minlength=C)
    assert np.array_equal(child_sum[~leaf], size[~leaf].astype(np.float64))
    assert np.array_equal(np.sort(d["order"]), np.arange(n))
    lc = np.repeat(np.nonzero(leaf)[0], size[leaf])
    idx = np.concatenate([d["order"][b:e] for b, e in zip(d["pt_begin"][leaf], d["pt_end"][leaf])])
    assert np.all(x[idx] >= d["mins"][lc]) and np.all(x[idx] <= d["maxs"][lc])
    assert st["m2l_pairs"] == sum(len(m) for m in d["m2l"])
    e = np.linalg.norm(a[tg] - ad, axis=1) / np.linalg.norm(ad, axis=1)
    rms = math.sqrt(np.mean(e * e))
    print(f"clustered 16M: FMM vs FP64 direct on 2048 particles RMS {rms:.3e} max {float(e.max()):.3e}")
    assert rms <= DIRECT_RMS_REL
