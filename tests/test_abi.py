"""The C-ABI library loads and exports every symbol include/vipp_gb300.h declares.

No compute call is made here (no GPU needed); gb_create must fail cleanly with
an error code when no device is present.
"""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vipp_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^GB_API\s+[\w\s\*]*?\b(gb_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    import vipp_gb300
    if not os.path.exists(vipp_gb300.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return vipp_gb300.load()


def test_header_declares_the_boundary():
    syms = declared_symbols()
    assert {"gb_create", "gb_upload", "gb_rk4_step", "gb_download", "gb_accel", "gb_tree_dump"} <= set(syms)


def test_library_exports_every_declared_symbol(lib):
    import vipp_gb300
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert set(declared_symbols()) == set(vipp_gb300.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", vipp_gb300.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(gb_\w+)$", out, re.M))
    assert set(declared_symbols()) <= exported


def test_version_string(lib):
    assert b"sm_103a" in lib.gb_version()


def test_create_without_gpu_reports_error(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import vipp_gb300
    cfg = vipp_gb300.GbConfig(4, 10, 0.01, 1.0, 1.0, 0, 0, 0)
    h = ctypes.c_void_p()
    rc = lib.gb_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc in (vipp_gb300.GB_ERR_NO_DEVICE, vipp_gb300.GB_ERR_CUDA)
    assert lib.gb_last_error(None)


def test_invalid_config_rejected_before_device(lib):
    import vipp_gb300
    h = ctypes.c_void_p()
    for bad in (vipp_gb300.GbConfig(0, 10, 0.01, 1, 1, 0, 0, 0), vipp_gb300.GbConfig(4, 0, 0.01, 1, 1, 0, 0, 0),
                vipp_gb300.GbConfig(11, 10, 0.01, 1, 1, 0, 0, 0), vipp_gb300.GbConfig(4, 10, -1.0, 1, 1, 0, 0, 0),
                vipp_gb300.GbConfig(4, 10, 0.01, 1, 1, 7, 0, 0)):
        assert lib.gb_create(ctypes.byref(bad), ctypes.byref(h)) == vipp_gb300.GB_ERR_INVALID


def test_null_handles_are_rejected(lib):
    """Every entry point taking a context or batch answers a NULL handle with
    GB_ERR_INVALID (or a neutral value) instead of touching memory."""
    import vipp_gb300
    INV = vipp_gb300.GB_ERR_INVALID
    buf = (ctypes.c_double * 6)()
    assert lib.gb_upload(None, buf, buf, 2) == INV
    assert lib.gb_download(None, buf, buf) == INV
    assert lib.gb_rk4_step(None, 1e-3) == INV
    assert lib.gb_accel(None, buf, None) == INV
    assert lib.gb_direct_accel(None, None, 0, buf) == INV
    assert lib.gb_sync(None) == INV
    assert lib.gb_get_stats(None, ctypes.byref(vipp_gb300.GbStats())) == INV
    assert lib.gb_get_conserved(None, ctypes.byref(vipp_gb300.GbConserved())) == INV
    assert lib.gb_init_plummer(None, 16, 0, 0.0) == INV
    assert lib.gb_tree_dump(None, *([None] * 17)) == INV
    assert lib.gb_enable_timing(None, 1) == INV
    assert lib.gb_kernel_times(None, None, None, 0) == INV
    assert lib.gb_set_config(None, ctypes.byref(vipp_gb300.GbConfig(4, 10, 0.01, 1, 1, 0, 0, 0))) == INV
    assert lib.gb_launch_count(None) == 0
    assert not lib.gb_stream(None)
    lib.gb_destroy(None)
    assert lib.gb_batch_upload(None, buf, buf) == INV
    assert lib.gb_batch_download(None, buf, buf) == INV
    assert lib.gb_batch_rk4_step(None, 1e-3) == INV
    assert not lib.gb_batch_system(None, 0)
    lib.gb_batch_destroy(None)


def test_batch_arguments_checked_before_device(lib):
    import vipp_gb300
    cfg = vipp_gb300.GbConfig(4, 10, 0.01, 1, 1, 0, 0, 0)
    b = ctypes.c_void_p()
    off = (ctypes.c_uint64 * 3)(0, 10, 5)  # decreasing
    assert lib.gb_batch_create(ctypes.byref(cfg), 2, off, None, ctypes.byref(b)) == vipp_gb300.GB_ERR_INVALID
    assert b"must not decrease" in lib.gb_batch_last_error(None)
    assert lib.gb_batch_create(ctypes.byref(cfg), 0, off, None, ctypes.byref(b)) == vipp_gb300.GB_ERR_INVALID
    assert lib.gb_batch_create(ctypes.byref(cfg), 2, None, None, ctypes.byref(b)) == vipp_gb300.GB_ERR_INVALID
    assert not b.value


def test_missing_library_fails_loudly(tmp_path):
    """No fallback: without the built CUDA library the binding raises (in a
    fresh interpreter, since this one has the library loaded already)."""
    import sys
    code = ("import sys; sys.path.insert(0, sys.argv[1]); import vipp_gb300; "
            "vipp_gb300.load(sys.argv[2])")
    r = subprocess.run([sys.executable, "-c", code, os.path.join(ROOT, "vipp-nbody-bench_gb300"),
                        str(tmp_path / "libvipp_gb300.so")], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "not built" in r.stderr
