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
