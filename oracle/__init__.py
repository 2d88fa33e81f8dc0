"""ORACLE — test infrastructure, not product code.

ctypes bindings for
  * ``liboracle.so``: the CPU restatement of the reference's gravity FMM path
    (oracle.hpp; every function cites the reference lines it restates), and
  * ``_ref/libvipp_ref.so``: the reference's own headers compiled unmodified
    behind a thin shim (ref_shim.cpp). It exists only where the reference
    sources are present; elsewhere ``ref()`` returns None.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use this module, always as the checker or the timed CPU
baseline, never as the thing measured on the GPU.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_ll_p = ctypes.POINTER(ctypes.c_longlong)
_c_int_p = ctypes.POINTER(ctypes.c_int)
_size = ctypes.c_size_t

_LIB = None
_REF = None
_REF_TRIED = False


def build(ref: bool = True) -> None:
    """Compile liboracle.so (and oracle/_ref when the reference is present)."""
    subprocess.run(["sh", os.path.join(HERE, "build_oracle.sh")], check=True)
    if ref:
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True)


def _dp(a):
    return a.ctypes.data_as(_c_dbl_p)


def _lp(a):
    return a.ctypes.data_as(_c_ll_p)


def _ip(a):
    return a.ctypes.data_as(_c_int_p)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref=False)
        _LIB = ctypes.CDLL(path)
        _LIB.orc_tree_build.restype = _size
        _LIB.orc_threads.restype = ctypes.c_int
        for f in ("orc_accel", "orc_accel_mode", "orc_rk4", "orc_rk4_mode", "orc_accel_sampled",
                  "orc_soft_correction_check"):
            getattr(_LIB, f).restype = ctypes.c_int
    return _LIB


def ref():
    """The compiled reference (None where its sources were not available)."""
    global _REF, _REF_TRIED
    if not _REF_TRIED:
        _REF_TRIED = True
        path = os.path.join(HERE, "_ref", "libvipp_ref.so")
        if os.path.exists(path):
            try:
                _REF = ctypes.CDLL(path)
                _REF.ref_tree_build.restype = _size
                _REF.ref_expansions.restype = _size
                _REF.ref_initialize.restype = ctypes.c_int
            except OSError:
                _REF = None
    return _REF


def _aos(a):
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)


class Impl:
    """One of the two CPU implementations with a common Python surface."""

    def __init__(self, handle, prefix):
        self.h = handle
        self.px = prefix

    def _f(self, name):
        return getattr(self.h, self.px + name)

    def accel(self, x, s, G, m, eps, p, mode=0):
        """One force evaluation. mode 0 is the reference's method; mode 1 the
        accurate mode (oracle only: far field times G plus the softening
        correction, oracle.hpp softening_correction)."""
        x = _aos(x)
        a = np.zeros_like(x)
        n = x.shape[0]
        if self.px == "orc_":
            rc = self.h.orc_accel_mode(_dp(x), _size(n), _size(s), ctypes.c_double(G), ctypes.c_double(m),
                                       ctypes.c_double(eps), ctypes.c_uint(p), ctypes.c_int(mode), _dp(a), None)
            if rc:
                raise RuntimeError("oracle accel failed")
        else:
            assert mode == 0, "the reference has only its own method"
            self.h.ref_accel(_dp(x), _size(n), _size(s), ctypes.c_double(G), ctypes.c_double(m),
                             ctypes.c_double(eps), ctypes.c_uint(p), _dp(a))
        return a

    def rk4(self, x, v, s, G, m, eps, dt, p, steps=1, mode=0):
        x = _aos(x).copy()
        v = _aos(v).copy()
        n = x.shape[0]
        args = (_dp(x), _dp(v), _size(n), ctypes.c_double(G), ctypes.c_double(m), ctypes.c_double(eps),
                ctypes.c_double(dt), _size(s), ctypes.c_uint(p), ctypes.c_int(steps))
        if mode:
            assert self.px == "orc_", "the reference has only its own method"
            rc = self.h.orc_rk4_mode(*args, ctypes.c_int(mode))
        else:
            rc = self._f("rk4")(*args)
        if self.px == "orc_" and rc:
            raise RuntimeError("oracle rk4 failed")
        return x, v

    def direct_rk4(self, x, v, G, m, eps, dt, steps=1):
        x = _aos(x).copy()
        v = _aos(v).copy()
        n = x.shape[0]
        f = self.h.orc_direct_rk4 if self.px == "orc_" else self.h.ref_naive_rk4
        f(_dp(x), _dp(v), _size(n), ctypes.c_double(G), ctypes.c_double(m), ctypes.c_double(eps),
          ctypes.c_double(dt), ctypes.c_int(steps))
        return x, v

    def P(self, nmax, x):
        out = np.zeros((nmax + 1) * (nmax + 1))
        self._f("P")(ctypes.c_uint(nmax), ctypes.c_double(x), _dp(out))
        return out.reshape(nmax + 1, nmax + 1)

    def DP(self, nmax, theta):
        out = np.zeros((nmax + 1) * (nmax + 1))
        self._f("DP")(ctypes.c_uint(nmax), ctypes.c_double(theta), _dp(out))
        return out.reshape(nmax + 1, nmax + 1)

    def Y(self, nmax, theta, phi):
        """Y[n, m + nmax] complex."""
        out = np.zeros((nmax + 1) * (2 * nmax + 1) * 2)
        self._f("Y")(ctypes.c_uint(nmax), ctypes.c_double(theta), ctypes.c_double(phi), _dp(out))
        out = out.reshape(nmax + 1, 2 * nmax + 1, 2)
        return out[..., 0] + 1j * out[..., 1]

    def tree(self, x, s):
        """Tree + lists as plain arrays (cell numbering of this implementation)."""
        x = _aos(x)
        n = x.shape[0]
        nc = int(self._f("tree_build")(_dp(x), _size(n), _size(s)))
        parent = np.zeros(nc, np.int64)
        level = np.zeros(nc, np.int32)
        first_child = np.zeros(nc, np.int64)
        mins = np.zeros((nc, 3))
        maxs = np.zeros((nc, 3))
        pt_off = np.zeros(nc + 1, np.int64)
        pts = np.zeros(max(n, 1), np.int64)
        sizes = np.zeros((nc, 3), np.int64)
        self._f("tree_fetch")(_lp(parent), _ip(level), _lp(first_child), _dp(mins), _dp(maxs), _lp(pt_off),
                              _lp(pts), _lp(sizes))
        tot = sizes.sum(axis=0)
        m2l = np.zeros(max(tot[0], 1), np.int64)
        p2p = np.zeros(max(tot[1], 1), np.int64)
        coll = np.zeros(max(tot[2], 1), np.int64)
        self._f("tree_lists")(_lp(m2l), _lp(p2p), _lp(coll))

        def split(arr, sz):
            off = np.concatenate([[0], np.cumsum(sz)])
            return [arr[off[i]:off[i + 1]] for i in range(len(sz))]

        return dict(parent=parent, level=level, first_child=first_child, mins=mins, maxs=maxs,
                    pts=[pts[pt_off[i]:pt_off[i + 1]] for i in range(nc)],
                    m2l=split(m2l, sizes[:, 0]), p2p=split(p2p, sizes[:, 1]), coll=split(coll, sizes[:, 2]))


def oracle() -> Impl:
    return Impl(lib(), "orc_")


def reference():
    r = ref()
    return None if r is None else Impl(r, "ref_")


def threads() -> int:
    return int(lib().orc_threads())


def set_threads(n: int) -> None:
    lib().orc_set_threads(ctypes.c_int(n))


def direct_accel(x, G, m, eps, targets=None):
    """FP64 direct softened sum (OpenMP) for the given targets (all if None)."""
    x = _aos(x)
    n = x.shape[0]
    if targets is None:
        a = np.zeros_like(x)
        lib().orc_direct_accel(_dp(x), _size(n), ctypes.c_double(G), ctypes.c_double(m), ctypes.c_double(eps),
                               None, _size(0), _dp(a))
    else:
        t = np.ascontiguousarray(targets, dtype=np.int64)
        a = np.zeros((len(t), 3))
        lib().orc_direct_accel(_dp(x), _size(n), ctypes.c_double(G), ctypes.c_double(m), ctypes.c_double(eps),
                               _lp(t), _size(len(t)), _dp(a))
    return a


def direct_phi(x, G, m, eps, targets=None):
    """FP64 direct softened potential -G m sum_{j != i} (r^2 + eps^2)^-1/2 (OpenMP)."""
    x = _aos(x)
    n = x.shape[0]
    t = None if targets is None else np.ascontiguousarray(targets, dtype=np.int64)
    phi = np.zeros(n if t is None else len(t))
    lib().orc_direct_phi(_dp(x), _size(n), ctypes.c_double(G), ctypes.c_double(m), ctypes.c_double(eps),
                         None if t is None else _lp(t), _size(0 if t is None else len(t)), _dp(phi))
    return phi


def plummer_reference(n, eps, seed):
    """Problem::initialize (problem.hpp:188-211) restated: (x, v) AoS."""
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    lib().orc_plummer_reference(_size(n), ctypes.c_double(eps), ctypes.c_ulonglong(seed), _dp(x), _dp(v))
    return x, v


def soft_correction_check(x, s, G, m, eps, targets):
    """(exact, expanded) far-field softening correction at the targets: the
    exact sum over the far source particles and the accurate mode's expansion
    of it (oracle.hpp softening_correction)."""
    x = _aos(x)
    t = np.ascontiguousarray(targets, dtype=np.int64)
    ex = np.zeros((len(t), 3))
    ap = np.zeros((len(t), 3))
    rc = lib().orc_soft_correction_check(_dp(x), _size(x.shape[0]), _size(s), ctypes.c_double(G), ctypes.c_double(m),
                                         ctypes.c_double(eps), _lp(t), _size(len(t)), _dp(ex), _dp(ap))
    if rc:
        raise RuntimeError("oracle correction check failed")
    return ex, ap


def curve_fit(e, t):
    e = np.ascontiguousarray(e, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    a = ctypes.c_double()
    c = ctypes.c_double()
    lib().orc_curve_fit(_dp(e), _dp(t), _size(len(e)), ctypes.byref(a), ctypes.byref(c))
    return a.value, c.value


def kat(which):
    out = np.zeros(6)
    lib().orc_kat(ctypes.c_int(which), _dp(out))
    return out


def accel_sampled(x, s, G, m, eps, p, stride):
    """Timed sample of one FMM evaluation; see orc_accel_sampled."""
    x = _aos(x)
    times = np.zeros(3)
    counts = np.zeros(6, np.int64)
    rc = lib().orc_accel_sampled(_dp(x), _size(x.shape[0]), _size(s), ctypes.c_double(G), ctypes.c_double(m),
                                 ctypes.c_double(eps), ctypes.c_uint(p), _size(stride), _dp(times), _lp(counts))
    if rc:
        raise RuntimeError("oracle sampled accel failed")
    return times, counts
