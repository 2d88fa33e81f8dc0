"""Tracing: the library's NVTX ranges, seen through an NVTX injection library
(tests/cpp/nvtx_recorder.c) that records domains and push/pop ranges.

Every C-ABI entry point that queues GPU work opens its range before it checks
its arguments, so calls with a NULL handle exercise the ranges without a GPU:
the domain `vipp_gb300`, one balanced push/pop per call, named after the call.
The kernel-class ranges (tree, m2l, p2p, ...) need a GPU; an ncu capture
filtered on the `m2l` range (ncu --nvtx --nvtx-include 'vipp_gb300@m2l]')
selects exactly that class's kernels."""
import os
import shutil
import subprocess
import sys

import pytest

import vipp_gb300

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALLS = ["gb_rk4_step", "gb_upload", "gb_download", "gb_accel", "gb_sync", "gb_batch_rk4_step",
         "gb_checkpoint_save", "gb_checkpoint_load"]

DRIVER = r"""
import ctypes, sys
lib = ctypes.CDLL(sys.argv[1])
vp, d = ctypes.c_void_p, ctypes.c_double
lib.gb_rk4_step.argtypes = [vp, d]
lib.gb_upload.argtypes = [vp, vp, vp, ctypes.c_size_t]
lib.gb_download.argtypes = [vp, vp, vp]
lib.gb_accel.argtypes = [vp, vp, vp]
lib.gb_sync.argtypes = [vp]
lib.gb_batch_rk4_step.argtypes = [vp, d]
lib.gb_checkpoint_save.argtypes = [vp, ctypes.c_char_p, d]
lib.gb_checkpoint_load.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp]
rcs = [lib.gb_rk4_step(None, 1e-3), lib.gb_upload(None, None, None, 0), lib.gb_download(None, None, None),
       lib.gb_accel(None, None, None), lib.gb_sync(None), lib.gb_batch_rk4_step(None, 1e-3),
       lib.gb_checkpoint_save(None, b"x", 0.0), lib.gb_checkpoint_load(None, b"x", 0, None)]
assert all(rc == 1 for rc in rcs), rcs
"""


def cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def test_entry_points_open_named_ranges_in_the_library_domain(tmp_path):
    if not os.path.exists(vipp_gb300.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    inc = cuda_include()
    if not os.path.exists(os.path.join(inc, "nvtx3", "nvToolsExt.h")):
        pytest.skip("no NVTX3 headers")
    so = str(tmp_path / "libnvtx_recorder.so")
    subprocess.run(["gcc", "-shared", "-fPIC", "-O1", "-I", inc, os.path.join(ROOT, "tests", "cpp", "nvtx_recorder.c"),
                    "-o", so], check=True)
    rec = tmp_path / "ranges.txt"
    env = dict(os.environ, NVTX_INJECTION64_PATH=so, NVTX_RECORD_FILE=str(rec))
    r = subprocess.run([sys.executable, "-c", DRIVER, vipp_gb300.LIB_PATH], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = rec.read_text().splitlines()
    assert "domain vipp_gb300" in lines
    ours = [ln for ln in lines if ln.startswith(("push vipp_gb300", "pop vipp_gb300"))]
    # one push and its pop per call, in call order
    expect = []
    for c in CALLS:
        expect += [f"push vipp_gb300 {c}", "pop vipp_gb300"]
    assert ours == expect, ours
