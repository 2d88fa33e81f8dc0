"""C++ drop-in adapter (include/gravity/solver_gb300.hpp) driven like the
reference's benchmark drives a Solver; see tests/cpp/test_solver_gb300.cpp."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vipp-nbody-bench_gb300")


def build(out, src="test_solver_gb300.cpp"):
    lib = os.path.join(PKG, "lib")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(PKG, "include"), os.path.join(ROOT, "tests", "cpp", src), "-L", lib,
           "-lvipp_gb300", f"-Wl,-rpath,{lib}", "-o", out]
    subprocess.run(cmd, check=True)


def test_adapter_compiles(tmp_path):
    import vipp_gb300
    vipp_gb300.load()
    build(str(tmp_path / "t"))


@pytest.mark.gpu
def test_adapter_runs_like_reference_solver(tmp_path):
    exe = str(tmp_path / "t")
    build(exe)
    r = subprocess.run([exe], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout


def test_benchmark_driver_compiles(tmp_path):
    import vipp_gb300
    vipp_gb300.load()
    build(str(tmp_path / "b"), "test_benchmark_gb300.cpp")


@pytest.mark.gpu
def test_benchmark_driver_accepts_and_rejects_like_reference(tmp_path):
    """benchmark_gb300.hpp: E(T) = alpha T^c fit and the reference's PASS rule."""
    exe = str(tmp_path / "b")
    build(exe, "test_benchmark_gb300.cpp")
    r = subprocess.run([exe], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
