"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's gravity headers compiled unmodified (oracle/_ref, built by
oracle/build_ref.sh from the reference sources) on small seeded inputs and
stores inputs and outputs as .npz files:

  tree_*.npz   particle positions, the reference's octree (cell parent, level,
               first child, box, member list) and calc_link lists
               (solver_ref.hpp:115-162), FMM accelerations
               (SolverRef::acceleration) and one RK4 step (runge_kutta)
  tree_plummer16384_s64_p8.npz, tree_uniform16384_s64_p6.npz
               the same at the headline orders and leaf capacity (Plummer
               sphere from Problem::initialize with eps = 0.005, p = 8, s = 64;
               unit cube with eps = 1e-3, p = 6, s = 64); positions are not
               stored but regenerated (the oracle's bit-identical restatement
               of Problem::initialize, or numpy's PCG64 stream) and checked
               against a stored checksum
  traj_plummer16384_s32_p4.npz
               the reference's CPU-runnable case run to its end: Plummer
               N = 16,384 (Problem::initialize, seed 0), s = 32, eps = 0.01,
               p = 4, ten RK4 steps of dt = 1e-3 (solver_ref.hpp:36-104);
               final positions and velocities
  kat.npz      special functions P, DP, Y (fmm.hpp:20-194) at the angles the
               reference's own tests use, the P2M/M2M/L known answers of
               test_fmm.cpp, Problem pieces (problem.hpp:250-292), curve fits
               (benchmark.hpp:198-242) and the direct-sum two-body RK4
               (solver_ref_naive.hpp)

Usage (needs the reference sources, i.e. the development container):
    python tests/golden/make_golden.py [small] [headline] [trajectory]
(no argument: all groups)
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def flat(lists):
    off = np.zeros(len(lists) + 1, np.int64)
    off[1:] = np.cumsum([len(a) for a in lists])
    data = np.concatenate([np.asarray(a, np.int64) for a in lists]) if off[-1] else np.zeros(0, np.int64)
    return off, data


def ref_problem(n, s, eps, p, seed, has_eps=True):
    r = O.ref()
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    e = ctypes.c_double()
    dt = ctypes.c_double()
    m = ctypes.c_double()
    rc = r.ref_initialize(ctypes.c_size_t(n), ctypes.c_size_t(s), ctypes.c_double(eps), int(has_eps), ctypes.c_uint(p),
                          ctypes.c_uint64(seed), O._dp(x), O._dp(v), ctypes.byref(e), ctypes.byref(dt), ctypes.byref(m))
    assert rc == 0
    return x, v, e.value, dt.value, m.value


def tree_case(name, x, v, s, p, eps, G=1.0, dt=1e-3):
    ref = O.reference()
    n = x.shape[0]
    m = 1.0 / n
    t = ref.tree(x, s)
    a = ref.accel(x, s, G, m, eps, p)
    x1, v1 = ref.rk4(x, v, s, G, m, eps, dt, p, 1)
    out = dict(x=x, v=v, s=s, p=p, eps=eps, G=G, m=m, dt=dt, parent=t["parent"], level=t["level"],
               first_child=t["first_child"], mins=t["mins"], maxs=t["maxs"], acc=a, x1=x1, v1=v1)
    for k in ("pts", "m2l", "p2p", "coll"):
        out[k + "_off"], out[k] = flat(t[k])
    np.savez_compressed(os.path.join(HERE, f"tree_{name}.npz"), **out)
    print(name, "cells", len(t["parent"]), "depth", int(t["level"].max()))


def checksum(a):
    """Order-sensitive FP64 checksum of an array (exact for identical arrays)."""
    a = np.ascontiguousarray(a, np.float64).ravel()
    return np.array([a.sum(), (a * np.arange(1, a.size + 1)).sum(), a.size], np.float64)


def big_case(name, gen, x, s, p, eps, G=1.0):
    """Tree, lists and FP64 accelerations of the reference; positions replaced
    by their generator description and checksum; integer arrays as int32."""
    ref = O.reference()
    n = x.shape[0]
    m = 1.0 / n
    t = ref.tree(x, s)
    a = ref.accel(x, s, G, m, eps, p)
    out = dict(gen=np.array(gen, np.float64), x_sum=checksum(x), s=s, p=p, eps=eps, G=G, m=m, dt=0.0,
               parent=t["parent"].astype(np.int32), level=t["level"].astype(np.int32),
               first_child=t["first_child"].astype(np.int32), mins=t["mins"], maxs=t["maxs"], acc=a)
    for k in ("pts", "m2l", "p2p", "coll"):
        off, data = flat(t[k])
        out[k + "_off"], out[k] = off.astype(np.int32), data.astype(np.int32)
    np.savez_compressed(os.path.join(HERE, f"tree_{name}.npz"), **out)
    print(name, "cells", len(t["parent"]), "depth", int(t["level"].max()))


def headline():
    # gen = [kind, n, eps or seed, seed]: kind 0 = Problem::initialize(n, eps, seed), 1 = PCG64(seed) unit cube
    x, _, eps, _, _ = ref_problem(16384, 64, 0.005, 8, 2)
    big_case("plummer16384_s64_p8", [0, 16384, 0.005, 2], x, 64, 8, eps)
    xu = np.random.default_rng(1).random((16384, 3))
    big_case("uniform16384_s64_p6", [1, 16384, 0, 1], xu, 64, 6, 1e-3)


def trajectory():
    n, s, p, eps, dt, steps = 16384, 32, 4, 0.01, 1e-3, 10
    x, v, e, _, m = ref_problem(n, s, eps, p, 0)
    assert e == eps and m == 1.0 / n
    x10, v10 = O.reference().rk4(x, v, s, 1.0, m, eps, dt, p, steps)
    np.savez_compressed(os.path.join(HERE, "traj_plummer16384_s32_p4.npz"), gen=np.array([0, n, eps, 0], np.float64),
                        x_sum=checksum(x), v_sum=checksum(v), s=s, p=p, eps=eps, G=1.0, m=m, dt=dt, steps=steps,
                        x10=x10, v10=v10)
    print("trajectory written")


def main(groups):
    if O.ref() is None:
        O.build(ref=True)
    assert O.ref() is not None, "reference build (oracle/_ref) unavailable"
    if "headline" in groups:
        headline()
    if "trajectory" in groups:
        trajectory()
    if "small" in groups:
        small()


def small():
    ref = O.reference()
    rng = np.random.default_rng(20260101)

    x, v, eps, _, _ = ref_problem(2000, 8, 0.01, 4, 0)
    tree_case("plummer2000_s8_p4", x, v, 8, 4, eps)
    x, v, eps, _, _ = ref_problem(3000, 4, 0.005, 6, 3)
    tree_case("plummer3000_s4_p6", x, v, 4, 6, eps)
    xu = rng.random((1500, 3))
    tree_case("uniform1500_s16_p3", xu, np.zeros_like(xu), 16, 3, 1e-3)
    c1 = 0.3 + 0.02 * rng.standard_normal((600, 3))
    c2 = 0.7 + 0.05 * rng.standard_normal((500, 3))
    bg = rng.random((100, 3))
    xc = np.concatenate([c1, c2, bg])
    tree_case("cluster1200_s6_p5", xc, 0.1 * rng.standard_normal(xc.shape), 6, 5, 1e-3)
    # tree shapes of gravity/test/test_octree.cpp and boundary sizes around T = floor(sqrt(8) s)
    tree_case("octree3", np.array([[1., 1, 1], [-1, -1, -1], [1, -1, 1]]), np.zeros((3, 3)), 1, 2, 0.01)
    tree_case("octree4", np.array([[4., 4, 4], [-4, -4, -4], [2, 2, 2], [3, 3, 3]]), np.zeros((4, 3)), 1, 2, 0.01)
    xt = rng.random((28, 3))  # s = 10: T = 28 -> root stays a leaf
    tree_case("root_leaf28_s10", xt, np.zeros_like(xt), 10, 3, 0.01)
    xt = rng.random((29, 3))  # one more particle splits the root
    tree_case("split29_s10", xt, np.zeros_like(xt), 10, 3, 0.01)
    # coordinates on the mid-planes of the root box: ties go to the upper half
    g = np.array([[i, j, k] for i in (-1., 0., 1.) for j in (-1., 0., 1.) for k in (-1., 0., 1.)])
    tree_case("midplane27_s1", g, np.zeros_like(g), 1, 2, 0.1)

    kat = {}
    for xv in (-1.0, 0.0, 1.0, 0.3):
        kat[f"P5_{xv}"] = ref.P(5, xv)
    for th in (0.0, np.pi / 4, np.pi / 2, 1.1):
        kat[f"Y5_{th:.6f}"] = ref.Y(5, th, 0.0 if th != 1.1 else 0.7)
        kat[f"DP5_{th:.6f}"] = ref.DP(5, th)
    kat["Y16_0.7_1.1"] = ref.Y(16, 0.7, 1.1)
    lo = np.zeros(2)
    O.ref().ref_kat_L(O._dp(lo))
    kat["L11"] = lo
    parts = []
    for x0, q in ((1 / 8, 0.0), (1 / 27, 0.6), (0.5, 1.0)):
        r_, ve, P = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        O.ref().ref_problem_parts(ctypes.c_double(x0), ctypes.c_double(q), ctypes.byref(r_), ctypes.byref(ve),
                                  ctypes.byref(P))
        parts.append([x0, q, r_.value, ve.value, P.value])
    kat["problem_parts"] = np.array(parts)
    fits = []
    t = np.array([1., 2, 4, 8, 16])
    for e in ([0, 0, 0, 0, 0], [1, 2, 4, 8, 16], [2, 8, 32, 128, 512], [2, .5, .125, 1 / 32, 1 / 128],
              [3e-3, 2e-4, 1.1e-5, 7e-7, 4e-8]):
        e = np.array(e, float)
        al, c = ctypes.c_double(), ctypes.c_double()
        O.ref().ref_curve_fitting(O._dp(e), O._dp(t), ctypes.c_size_t(5), ctypes.byref(al), ctypes.byref(c))
        fits.append(list(e) + [al.value, c.value])
    kat["curve_fits"] = np.array(fits)
    x2 = np.array([[0., 0, 0], [10, 0, 0]])
    xr, vr = ref.direct_rk4(x2, np.zeros((2, 3)), 1.0, 1.0, 1e-4, 1.0, 1)
    kat["naive_rk4_x"], kat["naive_rk4_v"] = xr, vr
    xi, vi, e0, dt0, m0 = ref_problem(100, 10, 0.0, 4, 0, has_eps=False)
    kat["init100_x"], kat["init100_v"] = xi, vi
    kat["init100_eps_dt_m"] = np.array([e0, dt0, m0])
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **kat)
    print("kat written")


if __name__ == "__main__":
    main(sys.argv[1:] or ["small", "headline", "trajectory"])
