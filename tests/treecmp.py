"""Canonical comparison of trees and interaction lists.

Cells are compared by (level, path): path = the child offsets from the root,
3 bits per level, offset bit a = 1 for the lower half along axis a (the
reference's convention, octree.hpp:164). This makes trees numbered in
different orders (the reference appends children in insertion order, the GPU
numbers cells level by level) directly comparable, including list order.
"""
import numpy as np

GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden")


def checksum(a):
    """Order-sensitive FP64 checksum (the one tests/golden/make_golden.py stores)."""
    a = np.ascontiguousarray(a, np.float64).ravel()
    return np.array([a.sum(), (a * np.arange(1, a.size + 1)).sum(), a.size], np.float64)


def regenerate(gen):
    """Positions and velocities of a fixture that stores its generator instead:
    gen = [0, n, eps, seed] is the reference's Problem::initialize (problem.hpp:188-211)
    through the oracle's bit-identical restatement; [1, n, 0, seed] is numpy's
    PCG64 unit cube at rest."""
    kind, n, eps, seed = int(gen[0]), int(gen[1]), float(gen[2]), int(gen[3])
    if kind == 0:
        import oracle
        return oracle.plummer_reference(n, eps, seed)
    x = np.random.default_rng(seed).random((n, 3))
    return x, np.zeros_like(x)


def load_case(name):
    z = np.load(f"{GOLDEN}/tree_{name}.npz")
    d = {k: z[k] for k in z.files}
    if "gen" in d:
        d["x"], d["v"] = regenerate(d["gen"])
        assert np.array_equal(checksum(d["x"]), d["x_sum"]), f"{name}: regenerated positions differ"

    def unflat(k):
        off, data = d[k + "_off"], d[k]
        return [data[off[i]:off[i + 1]] for i in range(len(off) - 1)]

    for k in ("pts", "m2l", "p2p", "coll"):
        d[k] = unflat(k)
    for k in ("s", "p"):
        d[k] = int(d[k])
    for k in ("eps", "G", "m", "dt"):
        d[k] = float(d[k])
    return d


def ref_keys(parent, first_child):
    """(level, path) of every cell of a reference-numbered tree."""
    n = len(parent)
    keys = [None] * n
    keys[0] = (0, 0)
    for c in range(1, n):  # parents precede children in the reference numbering
        p = int(parent[c])
        o = c - int(first_child[p])
        lv, pa = keys[p]
        keys[c] = (lv + 1, (pa << 3) | o)
    return keys


def canon_ref(t):
    """Reference/oracle tree dict -> {key: record}. p2p lists are full (inherited)."""
    keys = ref_keys(t["parent"], t["first_child"])
    out = {}
    for c, k in enumerate(keys):
        out[k] = dict(min=tuple(t["mins"][c]), max=tuple(t["maxs"][c]), leaf=int(t["first_child"][c]) < 0,
                      pts=tuple(int(i) for i in t["pts"][c]) if int(t["first_child"][c]) < 0 else (),
                      m2l=tuple(keys[int(u)] for u in t["m2l"][c]),
                      p2p=tuple(keys[int(u)] for u in t["p2p"][c]),
                      coll=tuple(keys[int(u)] for u in t["coll"][c]))
    return out


def canon_gpu(d):
    """GPU tree dump -> {key: record} with full p2p lists rebuilt from the own entries."""
    C = len(d["level"])
    keys = [(int(d["level"][c]), int(d["path"][c])) for c in range(C)]
    full = [None] * C
    for c in range(C):  # parents have smaller numbers
        p = int(d["parent"][c])
        own = tuple(keys[int(u)] for u in d["p2p_own"][c])
        full[c] = (full[p] if p >= 0 else ()) + own
    out = {}
    for c in range(C):
        leaf = int(d["first_child"][c]) < 0
        out[keys[c]] = dict(min=tuple(d["mins"][c]), max=tuple(d["maxs"][c]), leaf=leaf,
                            pts=tuple(int(i) for i in d["order"][d["pt_begin"][c]:d["pt_end"][c]]) if leaf else (),
                            m2l=tuple(keys[int(u)] for u in d["m2l"][c]), p2p=full[c],
                            coll=tuple(keys[int(u)] for u in d["coll"][c]))
    return out


def diff_trees(a, b, limit=5):
    """List of human-readable differences (empty when identical)."""
    msgs = []
    ka, kb = set(a), set(b)
    if ka != kb:
        msgs.append(f"cell sets differ: only-left {sorted(ka - kb)[:limit]} only-right {sorted(kb - ka)[:limit]}")
        return msgs
    for k in sorted(ka):
        for f in ("min", "max", "leaf", "pts", "m2l", "p2p", "coll"):
            if a[k][f] != b[k][f]:
                msgs.append(f"cell {k} field {f}: {str(a[k][f])[:120]} != {str(b[k][f])[:120]}")
                if len(msgs) >= limit:
                    return msgs
    return msgs


def rel_err(a, b):
    """Per-particle |a-b|/|b|."""
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
