"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs on any host (oracle vs golden fixtures, host logic, the
C-ABI library's exports); `-m gpu` runs the CUDA parity tests through the
C-ABI on a GB300.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vipp-nbody-bench_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
