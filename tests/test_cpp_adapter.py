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
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
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


def test_benchmark_driver_writes_reference_print_files(tmp_path):
    """Built with ENABLE_PRINT, the benchmark driver writes before.csv and
    after<T>.csv (x,y,z per line, the stream's default 6-significant-digit
    format), the files of the reference's ENABLE_PRINT build. Host-only stub
    solvers: no GPU."""
    exe = str(tmp_path / "p")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(PKG, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_benchmark_print.cpp"), "-o", exe]
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    x0 = [(0.125, -1.5, 2.0), (1.0 / 3.0, 1e-7, -123456.789), (0.0, 2.5e10, -0.0)]

    def lines(pts):
        return ["%g,%g,%g" % p for p in pts]

    assert open(tmp_path / "before.csv").read().splitlines() == lines(x0)
    for t in (1, 2, 4):
        moved = [(x + t * 1e-3, y, z) for x, y, z in x0]
        assert open(tmp_path / f"after{t}.csv").read().splitlines() == lines(moved), t
