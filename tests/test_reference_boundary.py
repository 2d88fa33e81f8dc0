"""The boundary against the reference's own types and driver, compiled and
linked (no GPU needed; the programs are not run):

  * tests/cpp/test_reference_types.cpp: gravity::SolverGB300 instantiated with
    gravity::Problem and gravity::Vector (gravity/include/problem.hpp:32-302);
  * the reference's own gravity/src/main.cpp, unmodified, with the Solver
    alias (gravity/include/solver.hpp:6-9) pointed at SolverGB300 by a
    replacement solver.hpp found first on the include path (SHIM below), so
    Benchmark::benchmark
    (benchmark.hpp:91-175) drives it; also with GRAVITY_FLOAT and with
    ENABLE_DIFFERENT_PRECISION (benchmark_different_precision, benchmark.hpp:33-87).

Runs where the reference sources are present (the directory oracle/build_ref.sh
read them from, recorded in oracle/_ref/REFERENCE_DIR); skipped elsewhere.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vipp-nbody-bench_gb300")
# the reference headers lean on transitive std includes (as oracle/build_ref.sh)
FORCE = [a for h in ("vector", "cmath", "complex", "optional", "tuple", "chrono", "functional", "algorithm", "iterator",
                     "limits", "variant", "stdexcept") for a in ("-include", h)]

SHIM = """#ifndef GRAVITY_SOLVER_HPP
#define GRAVITY_SOLVER_HPP
#include <solver_ref.hpp>
#include <gravity/solver_gb300.hpp>
namespace gravity {
template <class M, class T, class X, class V, class A, class G>
using Solver = SolverGB300<M, T, X, V, A, G>;
}
#endif
"""


def reference_dir():
    f = os.path.join(ROOT, "oracle", "_ref", "REFERENCE_DIR")
    if not os.path.exists(f):
        return None
    d = open(f).read().strip()
    return d if os.path.isdir(os.path.join(d, "gravity", "include")) else None


@pytest.fixture(scope="module")
def ref():
    d = reference_dir()
    if d is None:
        pytest.skip("reference sources not present")
    import vipp_gb300
    vipp_gb300.load()
    return d


def compile_link(src, out, incs, defs=()):
    lib = os.path.join(PKG, "lib")
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", *FORCE, *[f"-D{d}" for d in defs]]
    for i in incs:
        cmd += ["-I", i]
    cmd += ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "include"), src, "-L", lib, "-lvipp_gb300",
            f"-Wl,-rpath,{lib}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(out)


def test_adapter_with_reference_problem_and_vector(ref, tmp_path):
    compile_link(os.path.join(ROOT, "tests", "cpp", "test_reference_types.cpp"), str(tmp_path / "types"),
                 [os.path.join(ref, "gravity", "include")])


@pytest.mark.parametrize("defs", [(), ("GRAVITY_FLOAT",), ("ENABLE_DIFFERENT_PRECISION",)])
def test_reference_main_with_gb300_solver_alias(ref, tmp_path, defs):
    shim = tmp_path / "shim"
    shim.mkdir()
    (shim / "solver.hpp").write_text(SHIM)
    # the shim's directory comes first, so main.cpp's <solver.hpp> is the alias above
    compile_link(os.path.join(ref, "gravity", "src", "main.cpp"), str(tmp_path / "main"),
                 [str(shim), os.path.join(ref, "gravity", "include")], defs)
