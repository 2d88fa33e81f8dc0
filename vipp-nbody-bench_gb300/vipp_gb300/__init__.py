"""Python binding of libvipp_gb300.so (the C-ABI in include/vipp_gb300.h).

``Solver`` mirrors the reference's Solver concept
(gravity/include/solver_ref.hpp:11-27): ``preprocess`` uploads the particles,
``solve`` runs one RK4 step of size ``problem.delta_t() / t`` and
``postprocess`` downloads the state. Errors are raised as RuntimeError, as
the reference throws std::runtime_error.

The compute path is the CUDA library only: importing this module does not
fall back to anything else. ``load()`` raises if the shared library is
missing, and every call that needs a GPU raises if none is present.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libvipp_gb300.so")

GB_OK, GB_ERR_INVALID, GB_ERR_NONFINITE, GB_ERR_DEPTH, GB_ERR_CUDA, GB_ERR_NO_DEVICE, GB_ERR_STATE, GB_ERR_CAPACITY = range(8)
PREC = {"fp64": 0, "mixed": 1}
MODE = {"ref": 0, "accurate": 1}
FLAG_P2P_NEWTON = 1
FLAG_M2L_CUDA_CORES = 2
FLAG_SERIAL = 4
FLAG_NO_GRAPH = 8
FLAG_M2L_BF16 = 16
FLAG_BATCH_CONTEXTS = 32
CHECKPOINT_ANY_CONFIG = 1
TIMER_CLASSES = ("tree", "operators", "p2m_m2m", "m2l", "l2l_l2p", "p2p", "rk4", "soften")

# Every symbol include/vipp_gb300.h declares.
EXPORTS = ("gb_create", "gb_destroy", "gb_last_error", "gb_set_config", "gb_upload", "gb_download", "gb_rk4_step",
           "gb_accel", "gb_direct_accel", "gb_sync", "gb_get_stats", "gb_tree_dump", "gb_enable_timing",
           "gb_kernel_times", "gb_launch_count", "gb_version", "gb_stream", "gb_direct_accel_noalloc",
           "gb_get_conserved", "gb_init_plummer", "gb_batch_create", "gb_batch_destroy", "gb_batch_last_error",
           "gb_batch_upload", "gb_batch_download", "gb_batch_rk4_step", "gb_batch_size", "gb_batch_system",
           "gb_set_tuning", "gb_get_tuning", "gb_tuning_lookup", "gb_init_clustered", "gb_batch_init_plummer",
           "gb_batch_is_forest", "gb_batch_forest", "gb_batch_init_plummer_at", "gb_batch_accel", "gb_batch_conserved", "gb_batch_stats", "gb_batch_launch_count",
           "gb_checkpoint_write", "gb_checkpoint_read", "gb_checkpoint_save", "gb_checkpoint_load",
           "gb_batch_checkpoint_save", "gb_batch_checkpoint_load")
TUNING_FIELDS = ("p2p_blocks", "p2p_blocks_conc", "p2p_slice", "m2l_ctas_pct", "serial", "leaf_s", "p2p_occupancy")
TUNING_DEFAULT = {"p2p_blocks": 8, "p2p_blocks_conc": 8, "p2p_slice": 8192, "m2l_ctas_pct": 100, "serial": 0,
                  "leaf_s": 0, "p2p_occupancy": 8}


class GbConfig(ctypes.Structure):
    _fields_ = [("p", ctypes.c_int), ("s", ctypes.c_int), ("eps", ctypes.c_double), ("G", ctypes.c_double),
                ("m", ctypes.c_double), ("precision", ctypes.c_int), ("device", ctypes.c_int), ("flags", ctypes.c_int),
                ("mode", ctypes.c_int)]


class GbTuning(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in TUNING_FIELDS]


class GbConserved(ctypes.Structure):
    _fields_ = [("kinetic", ctypes.c_double), ("potential", ctypes.c_double), ("total", ctypes.c_double),
                ("momentum", ctypes.c_double * 3), ("angular_momentum", ctypes.c_double * 3)]


class GbStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("n", "ncells", "nleaves", "depth", "m2l_pairs", "p2p_pairs", "p2p_ranges", "retries",
                                                        "graph_steps", "direct_steps", "graph_captures", "steps")]


class GbCheckpointInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("nsys", ctypes.c_uint64), ("steps", ctypes.c_int64), ("t", ctypes.c_double),
                ("cfg", GbConfig), ("leaf_s", ctypes.c_int32)]


_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


def load(path: str | None = None):
    """Load the CUDA library (built by build.py). Raises if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libvipp_gb300.so not built ({path}); run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    lib.gb_create.argtypes = [ctypes.POINTER(GbConfig), ctypes.POINTER(vp)]
    lib.gb_destroy.argtypes = [vp]
    lib.gb_destroy.restype = None
    lib.gb_last_error.argtypes = [vp]
    lib.gb_last_error.restype = ctypes.c_char_p
    lib.gb_set_config.argtypes = [vp, ctypes.POINTER(GbConfig)]
    lib.gb_upload.argtypes = [vp, vp, vp, ctypes.c_size_t]
    lib.gb_download.argtypes = [vp, vp, vp]
    lib.gb_rk4_step.argtypes = [vp, ctypes.c_double]
    lib.gb_accel.argtypes = [vp, vp, vp]
    lib.gb_direct_accel.argtypes = [vp, vp, ctypes.c_size_t, vp]
    lib.gb_sync.argtypes = [vp]
    lib.gb_get_stats.argtypes = [vp, ctypes.POINTER(GbStats)]
    lib.gb_get_conserved.argtypes = [vp, ctypes.POINTER(GbConserved)]
    lib.gb_init_plummer.argtypes = [vp, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_double]
    lib.gb_tree_dump.argtypes = [vp] + [vp] * 17
    lib.gb_enable_timing.argtypes = [vp, ctypes.c_int]
    lib.gb_kernel_times.argtypes = [vp, vp, vp, ctypes.c_int]
    lib.gb_launch_count.argtypes = [vp]
    lib.gb_launch_count.restype = ctypes.c_int64
    lib.gb_version.restype = ctypes.c_char_p
    lib.gb_batch_create.argtypes = [ctypes.POINTER(GbConfig), ctypes.c_size_t, vp, vp, ctypes.POINTER(vp)]
    lib.gb_batch_destroy.argtypes = [vp]
    lib.gb_batch_destroy.restype = None
    lib.gb_batch_last_error.argtypes = [vp]
    lib.gb_batch_last_error.restype = ctypes.c_char_p
    lib.gb_batch_upload.argtypes = [vp, vp, vp]
    lib.gb_batch_download.argtypes = [vp, vp, vp]
    lib.gb_batch_rk4_step.argtypes = [vp, ctypes.c_double]
    lib.gb_batch_system.argtypes = [vp, ctypes.c_size_t]
    lib.gb_batch_system.restype = vp
    lib.gb_batch_is_forest.argtypes = [vp]
    lib.gb_batch_forest.argtypes = [vp]
    lib.gb_batch_forest.restype = vp
    lib.gb_batch_accel.argtypes = [vp, vp, vp]
    lib.gb_batch_conserved.argtypes = [vp, vp]
    lib.gb_batch_stats.argtypes = [vp, ctypes.POINTER(GbStats)]
    lib.gb_batch_launch_count.argtypes = [vp]
    lib.gb_batch_launch_count.restype = ctypes.c_int64
    lib.gb_stream.argtypes = [vp]
    lib.gb_stream.restype = vp
    lib.gb_direct_accel_noalloc.argtypes = [vp, ctypes.c_size_t, vp, ctypes.c_size_t, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, vp, vp]
    lib.gb_init_clustered.argtypes = [vp, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_double, vp]
    lib.gb_batch_init_plummer.argtypes = [vp, ctypes.c_uint64, ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
    lib.gb_batch_init_plummer_at.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_double, vp]
    ci = ctypes.POINTER(GbCheckpointInfo)
    lib.gb_checkpoint_write.argtypes = [ctypes.c_char_p, ci, vp, vp, vp, vp]
    lib.gb_checkpoint_read.argtypes = [ctypes.c_char_p, ci, vp, vp, ctypes.c_size_t, vp, vp, ctypes.c_size_t]
    lib.gb_checkpoint_save.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
    lib.gb_checkpoint_load.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.gb_batch_checkpoint_save.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
    lib.gb_batch_checkpoint_load.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.gb_set_tuning.argtypes = [vp, ctypes.POINTER(GbTuning)]
    lib.gb_get_tuning.argtypes = [vp, ctypes.POINTER(GbTuning)]
    lib.gb_tuning_lookup.argtypes = [ctypes.c_char_p, ctypes.POINTER(GbConfig), ctypes.c_size_t,
                                     ctypes.POINTER(GbTuning)]
    _LIB = lib
    return lib


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _aos(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, 3))


def tuning_lookup(path: str, n: int, p: int, precision: str = "mixed", mode: str = "ref", flags: int = 0):
    """The tuning-cache entry (dict) for a configuration and particle count, or
    None when the file has none (gb_tuning_lookup; no GPU needed)."""
    lib = load()
    cfg = GbConfig(p, 1, 0.0, 1.0, 1.0, PREC[precision], 0, flags, MODE[mode])
    t = GbTuning()
    rc = lib.gb_tuning_lookup(path.encode(), ctypes.byref(cfg), n, ctypes.byref(t))
    if rc == GB_ERR_STATE:
        return None
    if rc != GB_OK:
        raise GB300Error(rc, lib.gb_last_error(None).decode())
    return {k: int(getattr(t, k)) for k in TUNING_FIELDS}


class GB300Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gb error {code}: {msg}")
        self.code = code


def _config_dict(c: GbConfig) -> dict:
    return {"p": c.p, "s": c.s, "eps": c.eps, "G": c.G, "m": c.m, "precision": c.precision, "flags": c.flags,
            "mode": c.mode}


def checkpoint_write(path: str, x, v, p=4, s=10, eps=0.01, G=1.0, m=1.0, precision="fp64", flags=0, mode="ref",
                     seg=None, masses=None, steps=0, t=0.0, leaf_s=None):
    """Write a checkpoint from host arrays (gb_checkpoint_write; no GPU
    needed): x, v (n, 3), the configuration, segment offsets (nsys + 1, None
    for one system), per-system masses, the step count and time."""
    lib = load()
    x, v = _aos(x), _aos(v)
    n = x.shape[0]
    seg_a = None if seg is None else np.ascontiguousarray(seg, dtype=np.uint64)
    m_a = None if masses is None else np.ascontiguousarray(masses, dtype=np.float64)
    info = GbCheckpointInfo()
    info.n, info.nsys = n, 1 if seg_a is None else len(seg_a) - 1
    info.steps, info.t = int(steps), float(t)
    info.cfg = GbConfig(p, s, eps, G, m, PREC.get(precision, precision), 0, flags, MODE.get(mode, mode))
    info.leaf_s = s if leaf_s is None else int(leaf_s)
    rc = lib.gb_checkpoint_write(os.fsencode(path), ctypes.byref(info), _ptr(seg_a), _ptr(m_a), _ptr(x), _ptr(v))
    if rc != GB_OK:
        raise GB300Error(rc, lib.gb_last_error(None).decode())


def checkpoint_read(path: str, arrays: bool = True) -> dict:
    """Read a checkpoint (gb_checkpoint_read; no GPU needed): a dict with n,
    nsys, steps, t, config, leaf_s and, with arrays=True (check word
    verified), seg, masses, x and v."""
    lib = load()
    info = GbCheckpointInfo()
    fpath = os.fsencode(path)
    rc = lib.gb_checkpoint_read(fpath, ctypes.byref(info), None, None, 0, None, None, 0)
    if rc != GB_OK:
        raise GB300Error(rc, lib.gb_last_error(None).decode())
    out = {"n": int(info.n), "nsys": int(info.nsys), "steps": int(info.steps), "t": float(info.t),
           "config": _config_dict(info.cfg), "leaf_s": int(info.leaf_s)}
    if arrays:
        n, ns = out["n"], out["nsys"]
        seg, masses = np.zeros(ns + 1, np.uint64), np.zeros(ns)
        x, v = np.zeros((n, 3)), np.zeros((n, 3))
        rc = lib.gb_checkpoint_read(fpath, ctypes.byref(info), _ptr(seg), _ptr(masses), ns, _ptr(x), _ptr(v), n)
        if rc != GB_OK:
            raise GB300Error(rc, lib.gb_last_error(None).decode())
        out.update(seg=seg, masses=masses, x=x, v=v)
    return out


class Solver:
    """One solver context on one GPU (see include/vipp_gb300.h)."""

    def __init__(self, p: int = 4, s: int = 10, eps: float = 0.01, G: float = 1.0, m: float = 1.0,
                 precision: str = "fp64", device: int = 0, flags: int = 0, mode: str = "ref"):
        self.lib = load()
        self.cfg = GbConfig(p, s, eps, G, m, PREC[precision], device, flags, MODE[mode])
        h = ctypes.c_void_p()
        rc = self.lib.gb_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(None).decode())
        self.h = h
        self.n = 0

    def _check(self, rc):
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_config(self, **kw):
        for k, v in kw.items():
            if k == "precision":
                v = PREC[v]
            if k == "mode" and isinstance(v, str):
                v = MODE[v]
            setattr(self.cfg, k, v)
        self._check(self.lib.gb_set_config(self.h, ctypes.byref(self.cfg)))

    def set_tuning(self, **kw):
        """Change launch/tree parameters (gb_set_tuning); unnamed ones keep their values."""
        t = GbTuning()
        self._check(self.lib.gb_get_tuning(self.h, ctypes.byref(t)))
        for k, v in kw.items():
            if k not in TUNING_FIELDS:
                raise KeyError(k)
            setattr(t, k, int(v))
        self._check(self.lib.gb_set_tuning(self.h, ctypes.byref(t)))

    def tuning(self) -> dict:
        t = GbTuning()
        self._check(self.lib.gb_get_tuning(self.h, ctypes.byref(t)))
        return {k: int(getattr(t, k)) for k in TUNING_FIELDS}

    # Solver concept -------------------------------------------------------
    def preprocess(self, x, v):
        x, v = _aos(x), _aos(v)
        self.n = x.shape[0]
        self._check(self.lib.gb_upload(self.h, _ptr(x), _ptr(v), self.n))

    def solve(self, dt: float):
        self._check(self.lib.gb_rk4_step(self.h, float(dt)))

    def postprocess(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        self._check(self.lib.gb_download(self.h, _ptr(x), _ptr(v)))
        return x, v

    # extras ----------------------------------------------------------------
    def upload_ptr(self, x_ptr: int, v_ptr: int, n: int):
        """preprocess from raw host pointers (e.g. pinned buffers)."""
        self.n = n
        self._check(self.lib.gb_upload(self.h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(v_ptr), n))

    def download_ptr(self, x_ptr: int, v_ptr: int):
        self._check(self.lib.gb_download(self.h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(v_ptr)))

    def accel(self, potential=False):
        """Accelerations (n, 3); with potential=True also the potentials (n,),
        a = -grad phi (the near field FP64, softened, i == j excluded)."""
        a = np.zeros((self.n, 3))
        if not potential:
            self._check(self.lib.gb_accel(self.h, _ptr(a), None))
            return a
        phi = np.zeros(self.n)
        self._check(self.lib.gb_accel(self.h, _ptr(a), _ptr(phi)))
        return a, phi

    def init_plummer(self, n, seed=0, r_max=0.0):
        """Generate the reference's Plummer sphere on the device (r_max = 0: the
        reference's radius cap from eps; r_max > 0: radii <= r_max)."""
        self._check(self.lib.gb_init_plummer(self.h, int(n), int(seed), float(r_max)))
        self.n = int(n)

    def init_clustered(self, n, seed=4, clusters=8, background=0.05, r_max=10.0):
        """Generate the adaptive-depth stress workload on the device
        (gb_init_clustered); returns the clusters' parameters as a dict of
        arrays: centres, radii, bulk, sizes."""
        prm = np.zeros(8 * clusters)
        self._check(self.lib.gb_init_clustered(self.h, int(n), int(seed), int(clusters), float(background),
                                               float(r_max), _ptr(prm)))
        self.n = int(n)
        q = prm.reshape(clusters, 8)
        return {"centres": q[:, :3].copy(), "radii": q[:, 3].copy(), "bulk": q[:, 4:7].copy(),
                "sizes": q[:, 7].astype(np.int64)}

    def conserved(self) -> dict:
        """Kinetic, potential and total energy, momentum and angular momentum
        of the current state (one FMM evaluation for the potential)."""
        c = GbConserved()
        self._check(self.lib.gb_get_conserved(self.h, ctypes.byref(c)))
        return {"kinetic": c.kinetic, "potential": c.potential, "total": c.total,
                "momentum": np.array(c.momentum[:]), "angular_momentum": np.array(c.angular_momentum[:])}

    def direct_accel(self, targets=None):
        if targets is None:
            a = np.zeros((self.n, 3))
            self._check(self.lib.gb_direct_accel(self.h, None, 0, _ptr(a)))
        else:
            t = np.ascontiguousarray(targets, dtype=np.int64)
            a = np.zeros((len(t), 3))
            self._check(self.lib.gb_direct_accel(self.h, _ptr(t), len(t), _ptr(a)))
        return a

    def sync(self):
        self._check(self.lib.gb_sync(self.h))

    def stats(self) -> dict:
        s = GbStats()
        self._check(self.lib.gb_get_stats(self.h, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in GbStats._fields_}

    def enable_timing(self, on=True):
        self._check(self.lib.gb_enable_timing(self.h, int(on)))

    def save_checkpoint(self, path: str, t: float = 0.0):
        """Write the state, step count and time t to a checkpoint file."""
        self._check(self.lib.gb_checkpoint_save(self.h, os.fsencode(path), float(t)))

    def load_checkpoint(self, path: str, any_config: bool = False) -> float:
        """Replace the state from a checkpoint (configuration checked unless
        any_config); returns the saved time."""
        t = ctypes.c_double()
        self._check(self.lib.gb_checkpoint_load(self.h, os.fsencode(path), CHECKPOINT_ANY_CONFIG if any_config else 0,
                                                ctypes.byref(t)))
        self.n = checkpoint_read(path, arrays=False)["n"]
        return t.value

    def kernel_times(self) -> dict:
        n = len(TIMER_CLASSES)
        ms = np.zeros(n)
        cnt = np.zeros(n, np.int64)
        self._check(self.lib.gb_kernel_times(self.h, _ptr(ms), _ptr(cnt), n))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(TIMER_CLASSES)}

    def stream_ptr(self) -> int:
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        return int(self.lib.gb_stream(self.h) or 0)

    def launch_count(self) -> int:
        return int(self.lib.gb_launch_count(self.h))

    def tree_dump(self) -> dict:
        """Tree and lists of the last force evaluation (see gb_tree_dump)."""
        nc = np.zeros(1, np.int64)
        ls = np.zeros(3, np.int64)
        nulls = [None] * 15
        self._check(self.lib.gb_tree_dump(self.h, _ptr(nc), _ptr(ls), *nulls))
        C = int(nc[0])
        level = np.zeros(C, np.int32)
        parent = np.zeros(C, np.int64)
        first_child = np.zeros(C, np.int64)
        path = np.zeros(C, np.uint64)
        bmin = np.zeros((C, 3))
        bmax = np.zeros((C, 3))
        pb = np.zeros(C, np.int64)
        pe = np.zeros(C, np.int64)
        order = np.zeros(max(self.n, 1), np.int64)
        m2l_off = np.zeros(C + 1, np.int64)
        m2l = np.zeros(max(int(ls[0]), 1), np.int64)
        p2p_off = np.zeros(C + 1, np.int64)
        p2p = np.zeros(max(int(ls[1]), 1), np.int64)
        coll_off = np.zeros(C + 1, np.int64)
        coll = np.zeros(max(int(ls[2]), 1), np.int64)
        self._check(self.lib.gb_tree_dump(self.h, _ptr(nc), _ptr(ls), _ptr(level), _ptr(parent), _ptr(first_child),
                                          _ptr(path), _ptr(bmin), _ptr(bmax), _ptr(pb), _ptr(pe), _ptr(order),
                                          _ptr(m2l_off), _ptr(m2l), _ptr(p2p_off), _ptr(p2p), _ptr(coll_off),
                                          _ptr(coll)))
        return dict(level=level, parent=parent, first_child=first_child, path=path, mins=bmin, maxs=bmax,
                    pt_begin=pb, pt_end=pe, order=order[:self.n],
                    m2l=[m2l[m2l_off[c]:m2l_off[c + 1]] for c in range(C)],
                    p2p_own=[p2p[p2p_off[c]:p2p_off[c + 1]] for c in range(C)],
                    coll=[coll[coll_off[c]:coll_off[c + 1]] for c in range(C)])


def version() -> str:
    return load().gb_version().decode()


def shard_systems(sizes, world: int) -> list:
    """Contiguous runs of systems for `world` ranks, balanced by particle count
    (the work of a force evaluation grows with N): rank r gets systems
    [start_r, end_r). Rank r's run ends at the system boundary nearest to
    (r + 1) / world of the total particle count."""
    sizes = np.asarray(sizes, dtype=np.int64)
    pre = np.concatenate([[0], np.cumsum(sizes)])
    total = int(pre[-1])
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        cut = min(int(np.searchsorted(pre, target, side="left")), len(sizes))
        if cut > 0 and abs(pre[cut - 1] - target) <= abs(pre[cut] - target):
            cut -= 1
        bounds.append(max(bounds[-1], cut))
    bounds.append(len(sizes))
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


class Batch:
    """Independent systems of uneven N advanced together (gb_batch_*):
    sizes[k] particles of system k, concatenated in x and v; masses[k] is the
    particle mass of system k. The forest form (default) runs every system in
    one context and one launch per kernel class; flags |= FLAG_BATCH_CONTEXTS
    gives every system a context of its own (same results)."""

    def __init__(self, sizes, p=4, s=32, eps=0.01, G=1.0, masses=None, precision="mixed", device=0, flags=0,
                 mode="ref"):
        self.lib = load()
        sizes = np.asarray(sizes, dtype=np.uint64)
        self.off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
        self.cfg = GbConfig(p, s, eps, G, 1.0, PREC[precision], device, flags, MODE[mode])
        m = None if masses is None else np.ascontiguousarray(masses, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = self.lib.gb_batch_create(ctypes.byref(self.cfg), len(sizes), _ptr(self.off), _ptr(m), ctypes.byref(h))
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_batch_last_error(None).decode())
        self.h = h
        self.n = int(self.off[-1])

    def _check(self, rc):
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_batch_last_error(self.h).decode())

    def upload(self, x, v):
        x, v = _aos(x), _aos(v)
        assert x.shape[0] == self.n and v.shape[0] == self.n
        self._check(self.lib.gb_batch_upload(self.h, _ptr(x), _ptr(v)))

    def init_plummer(self, seed=3, r_lo=0.5, r_hi=2.0, r_max=10.0, first=0):
        """Generate every system on the device (gb_batch_init_plummer_at): Plummer
        spheres of total mass 1 scaled to radii uniform in [r_lo, r_hi]; system
        k is system first + k of the seeded family. Returns the radii."""
        radii = np.zeros(len(self.off) - 1)
        self._check(self.lib.gb_batch_init_plummer_at(self.h, int(seed), int(first), float(r_lo), float(r_hi),
                                                      float(r_max), _ptr(radii)))
        return radii

    def step(self, dt):
        self._check(self.lib.gb_batch_rk4_step(self.h, float(dt)))

    def save_checkpoint(self, path: str, t: float = 0.0):
        """Write every system's state, the step count and time t to a checkpoint file."""
        self._check(self.lib.gb_batch_checkpoint_save(self.h, os.fsencode(path), float(t)))

    def load_checkpoint(self, path: str, any_config: bool = False) -> float:
        """Replace the state from a checkpoint of this batch's systems; returns the saved time."""
        t = ctypes.c_double()
        self._check(self.lib.gb_batch_checkpoint_load(self.h, os.fsencode(path),
                                                      CHECKPOINT_ANY_CONFIG if any_config else 0, ctypes.byref(t)))
        return t.value

    @property
    def forest(self) -> bool:
        return bool(self.lib.gb_batch_is_forest(self.h))

    def accel(self, potential=False):
        """Accelerations (and potentials) of every system, concatenated."""
        a = np.zeros((self.n, 3))
        phi = np.zeros(self.n) if potential else None
        self._check(self.lib.gb_batch_accel(self.h, _ptr(a), _ptr(phi)))
        return (a, phi) if potential else a

    def conserved(self) -> list:
        """Conserved quantities of every system (gb_batch_conserved)."""
        out = (GbConserved * (len(self.off) - 1))()
        self._check(self.lib.gb_batch_conserved(self.h, out))
        return [{"kinetic": c.kinetic, "potential": c.potential, "total": c.total, "momentum": list(c.momentum),
                 "angular_momentum": list(c.angular_momentum)} for c in out]

    def stats(self) -> dict:
        st = GbStats()
        self._check(self.lib.gb_batch_stats(self.h, ctypes.byref(st)))
        return {f: int(getattr(st, f)) for f, _ in GbStats._fields_}

    def launch_count(self) -> int:
        return int(self.lib.gb_batch_launch_count(self.h))

    def _forest_ctx(self):
        c = self.lib.gb_batch_forest(self.h)
        if not c:
            raise GB300Error(GB_ERR_INVALID, "kernel timing of a batch needs the forest form")
        return c

    def enable_timing(self, on=True):
        """Per-class kernel timers of the forest's context (Solver.enable_timing)."""
        c = self._forest_ctx()
        rc = self.lib.gb_enable_timing(c, 1 if on else 0)
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(c).decode())

    def kernel_times(self) -> dict:
        """{class: (ms, launches)} accumulated since the last call (forest form)."""
        c = self._forest_ctx()
        ms = np.zeros(len(TIMER_CLASSES))
        nl = np.zeros(len(TIMER_CLASSES), dtype=np.int64)
        rc = self.lib.gb_kernel_times(c, _ptr(ms), _ptr(nl), len(TIMER_CLASSES))
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(c).decode())
        return {k: (float(ms[i]), int(nl[i])) for i, k in enumerate(TIMER_CLASSES)}

    def download(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        self._check(self.lib.gb_batch_download(self.h, _ptr(x), _ptr(v)))
        return x, v

    def system_stats(self, k) -> dict:
        """Statistics of system k's own context (contexts form only)."""
        c = self.lib.gb_batch_system(self.h, k)
        if not c:
            raise GB300Error(GB_ERR_INVALID, "system_stats needs the contexts form (forest: stats())")
        st = GbStats()
        rc = self.lib.gb_get_stats(c, ctypes.byref(st))
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(c).decode())
        return {f: int(getattr(st, f)) for f, _ in GbStats._fields_}

    def system_accel(self, k):
        """Accelerations of system k at its current positions."""
        c = self.lib.gb_batch_system(self.h, k)
        if not c:
            return self.accel()[int(self.off[k]):int(self.off[k + 1])]
        n = int(self.off[k + 1] - self.off[k])
        a = np.zeros((n, 3))
        rc = self.lib.gb_accel(c, _ptr(a), None)
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(c).decode())
        return a

    def system_conserved(self, k) -> dict:
        """Conserved quantities of system k (gb_get_conserved on its context;
        the forest form: gb_batch_conserved)."""
        c = self.lib.gb_batch_system(self.h, k)
        if not c:
            return self.conserved()[k]
        out = GbConserved()
        rc = self.lib.gb_get_conserved(c, ctypes.byref(out))
        if rc != GB_OK:
            raise GB300Error(rc, self.lib.gb_last_error(c).decode())
        return {"kinetic": out.kinetic, "potential": out.potential, "total": out.total,
                "momentum": list(out.momentum), "angular_momentum": list(out.angular_momentum)}

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
