"""CPU check of the CUDA kernels' math (csrc/harmonics.cuh is host+device).

Builds tests/cpu_operator_check.cpp with g++ and runs one FMM evaluation with
the library's solid-harmonic recurrences, scaled real-basis M2M/M2L/L2L
matrices and ladder-operator L2P on the oracle's tree; the accelerations must
equal the oracle's restatement of the reference to FP64 rounding.
"""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("opcheck") / "opcheck")
    subprocess.run(["g++", "-std=c++17", "-O2", "-include", "array", os.path.join(HERE, "cpu_operator_check.cpp"),
                    "-o", out], check=True)
    return out


@pytest.mark.parametrize("n,s,p", [(3000, 8, 4), (2000, 4, 3), (4000, 16, 8), (1500, 6, 6)])
def test_operator_algebra_matches_oracle(exe, n, s, p):
    r = subprocess.run([exe, str(n), str(s), str(p)], capture_output=True, text=True, check=True)
    f = r.stdout.split()
    vals = dict(zip(f[0::2], f[1::2]))
    assert float(vals["yerr"]) < 1e-12
    assert float(vals["maxrel"]) < 1e-11
    assert float(vals["rms"]) < 1e-13
