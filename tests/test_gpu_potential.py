"""Potentials and conserved quantities (no counterpart in the reference, whose
Solver computes no potential). Checked against the oracle's FP64 direct sum and
against host sums of the same state.

Tolerances (written here):
  * FMM potential vs FP64 direct (softened, i != j), set by the expansion
    order (truncation; the far field is unsoftened as in the reference):
    p = 4 RMS <= 5e-4, max <= 1e-2 (measured RMS 2.2e-4); p = 8 RMS <= 1e-4,
    max <= 5e-4 (measured 2.9e-5, 9.4e-5);
  * mixed vs FP64 potential: RMS relative <= 1e-5;
  * kinetic energy, momentum, angular momentum vs numpy: 1e-12 relative;
    potential energy vs 1/2 m sum(phi) of gb_accel: 1e-12 relative;
  * FP64 RK4, 10 steps of dt = 1e-3 on 16,384 Plummer particles: relative
    total-energy change <= 1e-4.
"""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plummer16k():
    x, v = O.plummer_reference(16384, 0.01, 0)
    return x, v


def rel_rms(a, b):
    return math.sqrt(np.mean(((a - b) / b) ** 2)), float(np.max(np.abs((a - b) / b)))


@pytest.mark.parametrize("p,tol_rms,tol_max", [(4, 5e-4, 1e-2), (8, 1e-4, 5e-4)])
def test_fmm_potential_vs_direct(plummer16k, p, tol_rms, tol_max):
    import vipp_gb300
    x, v = plummer16k
    n = len(x)
    with vipp_gb300.Solver(p=p, s=32, eps=0.01, m=1.0 / n) as s:
        s.preprocess(x, v)
        a, phi = s.accel(potential=True)
        a2 = s.accel()
    ref = O.direct_phi(x, 1.0, 1.0 / n, 0.01)
    rms, mx = rel_rms(phi, ref)
    print(f"p={p}: potential vs direct RMS {rms:.3e} max {mx:.3e}")
    assert np.array_equal(a, a2)  # asking for the potential leaves the accelerations unchanged
    assert np.all(phi < 0)
    assert rms <= tol_rms and mx <= tol_max


def test_mixed_potential_vs_fp64(plummer16k):
    import vipp_gb300
    x, v = plummer16k
    n = len(x)
    out = {}
    for prec in ("fp64", "mixed"):
        with vipp_gb300.Solver(p=6, s=32, eps=0.01, m=1.0 / n, precision=prec) as s:
            s.preprocess(x, v)
            out[prec] = s.accel(potential=True)[1]
    rms, mx = rel_rms(out["mixed"], out["fp64"])
    print(f"mixed vs fp64 potential RMS {rms:.3e} max {mx:.3e}")
    assert rms <= 1e-5


def test_conserved_sums_match_host(plummer16k):
    import vipp_gb300
    x, v = plummer16k
    n = len(x)
    m = 1.0 / n
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=m, G=1.0) as s:
        s.preprocess(x, v)
        c = s.conserved()
        c2 = s.conserved()
        phi = s.accel(potential=True)[1]
    assert c["total"] == c2["total"]  # deterministic
    kin = 0.5 * m * np.sum(v * v)
    assert c["kinetic"] == pytest.approx(kin, rel=1e-12)
    assert c["potential"] == pytest.approx(0.5 * m * np.sum(phi), rel=1e-12)
    assert c["total"] == pytest.approx(c["kinetic"] + c["potential"], rel=1e-15)
    np.testing.assert_allclose(c["momentum"], m * v.sum(axis=0), rtol=1e-10, atol=1e-15)
    np.testing.assert_allclose(c["angular_momentum"], m * np.cross(x, v).sum(axis=0), rtol=1e-10, atol=1e-15)


def test_energy_drift_fp64_rk4(plummer16k):
    import vipp_gb300
    x, v = plummer16k
    n = len(x)
    with vipp_gb300.Solver(p=8, s=32, eps=0.01, m=1.0 / n) as s:
        s.preprocess(x, v)
        e0 = s.conserved()["total"]
        for _ in range(10):
            s.solve(1e-3)
        e1 = s.conserved()["total"]
    drift = abs(e1 - e0) / abs(e0)
    print(f"relative energy change over 10 RK4 steps: {drift:.3e} (E0 = {e0:.6f})")
    assert e0 < 0 and drift <= 1e-4


def test_potential_small_cases():
    import vipp_gb300
    x = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    with vipp_gb300.Solver(p=4, s=4, eps=0.1, m=0.5, G=2.0) as s:
        s.preprocess(x, np.zeros_like(x))
        _, phi = s.accel(potential=True)
    assert phi == pytest.approx([-1.0 / math.sqrt(1.01)] * 2, rel=1e-14)
    with vipp_gb300.Solver(p=4, s=4) as s:
        s.preprocess(np.zeros((0, 3)), np.zeros((0, 3)))
        c = s.conserved()
        assert c["total"] == 0
