"""GPU initial conditions (gb_init_plummer) against the reference's Plummer
model (problem.hpp:188-292). The reference draws from one mt19937_64 stream
through implementation-defined uniform distributions, so parity is
distributional. Tolerances: every Kolmogorov-Smirnov distance below its
0.1% critical value (one sample: 1.95/sqrt(n); two samples of n: 1.95 sqrt(2/n)).
"""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

N = 200_000
KS1 = 1.95 / math.sqrt(N)
KS2 = 1.95 * math.sqrt(2.0 / N)


def mass(r):
    return r ** 3 / (1 + r * r) ** 1.5


def ks_one(sample, cdf):
    s = np.sort(sample)
    f = cdf(s)
    k = np.arange(1, len(s) + 1) / len(s)
    return max(np.max(k - f), np.max(f - (k - 1.0 / len(s))))


def ks_two(a, b):
    a, b = np.sort(a), np.sort(b)
    grid = np.concatenate([a, b])
    return np.max(np.abs(np.searchsorted(a, grid, side="right") / len(a) - np.searchsorted(b, grid, side="right") / len(b)))


def q_cdf():
    g = np.linspace(0, 1, 200_001)
    pdf = g * g * (1 - g * g) ** 3.5
    c = np.concatenate([[0], np.cumsum((pdf[1:] + pdf[:-1]) / 2)])
    c /= c[-1]
    return lambda q: np.interp(q, g, c)


def generate(n, seed, eps=0.01, r_max=0.0):
    import vipp_gb300
    with vipp_gb300.Solver(p=4, s=32, eps=eps, m=1.0 / max(n, 1)) as s:
        s.init_plummer(n, seed, r_max)
        return s.postprocess()


def speeds_fraction(x, v):
    r = np.linalg.norm(x, axis=1)
    return np.linalg.norm(v, axis=1) / (math.sqrt(2.0) * (r * r + 1) ** -0.25)


@pytest.mark.parametrize("r_max", [0.0, 10.0])
def test_plummer_radii_speeds_directions(r_max):
    eps = 0.01
    x, v = generate(N, 7, eps, r_max)
    r = np.linalg.norm(x, axis=1)
    top = mass(r_max) if r_max > 0 else 1 - eps
    assert r.max() <= (r_max if r_max > 0 else (1 - eps) ** (1 / 3) / math.sqrt(1 - (1 - eps) ** (2 / 3))) * (1 + 1e-12)
    assert ks_one(r, lambda s: mass(s) / top) < KS1
    assert ks_one(speeds_fraction(x, v), q_cdf()) < KS1
    for w, nw in ((x, r), (v, np.linalg.norm(v, axis=1))):
        u = w[:, 0] / nw  # first component (1 - 2u) n: uniform on [-1, 1]
        assert ks_one(u, lambda s: (s + 1) / 2) < KS1
        phi = np.arctan2(w[:, 2], w[:, 1])  # azimuth uniform
        assert ks_one(phi, lambda s: (s + np.pi) / (2 * np.pi)) < KS1


def test_plummer_matches_reference_generator():
    """Two-sample comparison with the oracle's bit-identical restatement of
    the reference's Problem::initialize (same eps cap)."""
    eps = 0.01
    x, v = generate(N, 3, eps)
    xr, vr = O.plummer_reference(N, eps, 3)
    assert ks_two(np.linalg.norm(x, axis=1), np.linalg.norm(xr, axis=1)) < KS2
    assert ks_two(np.linalg.norm(v, axis=1), np.linalg.norm(vr, axis=1)) < KS2
    assert ks_two(x[:, 0], xr[:, 0]) < KS2 and ks_two(v[:, 2], vr[:, 2]) < KS2


def test_plummer_seeds_and_sizes():
    a = generate(10_000, 11)
    b = generate(10_000, 11)
    c = generate(10_000, 12)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])
    d = generate(20_000, 11)  # per-particle streams: a prefix does not depend on n
    assert np.array_equal(d[0][:10_000], a[0])
    assert generate(0, 1)[0].shape == (0, 3)


def test_generated_state_steps():
    import vipp_gb300
    n = 50_000
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n, precision="mixed") as s:
        s.init_plummer(n, 5)
        e0 = s.conserved()
        s.solve(1e-3)
        e1 = s.conserved()
    assert e0["total"] < 0 and abs(e1["total"] - e0["total"]) < 1e-5 * abs(e0["total"])
    assert -2 * e0["kinetic"] / e0["potential"] == pytest.approx(1.0, abs=0.05)  # virial equilibrium


def test_clustered_workload_on_the_device():
    """gb_init_clustered: the adaptive-depth stress workload. Background: the
    last round(0.05 n) particles, uniform in [0, 1)^3 (KS per axis) and at
    rest; cluster k: radii from its centre in units of its scale radius
    follow the Plummer mass profile capped at 10 (KS), its mean velocity is
    its bulk velocity, and its internal speeds scale as sqrt(m_k / a_k) (the
    speed fraction follows the Plummer distribution function's q law, KS);
    deterministic per seed."""
    import vipp_gb300
    n = 400_000
    with vipp_gb300.Solver(p=4, s=64, eps=1e-4, m=1.0 / n) as s:
        prm = s.init_clustered(n, seed=4)
        x, v = s.postprocess()
        prm2 = s.init_clustered(n, seed=4)
        x2, _ = s.postprocess()
        s.init_clustered(n, seed=5)
        x3, _ = s.postprocess()
    assert np.array_equal(x, x2) and not np.array_equal(x, x3)
    assert np.array_equal(prm["radii"], prm2["radii"])
    nbg = int(round(0.05 * n))
    bg = slice(n - nbg, n)
    assert np.all(v[bg] == 0) and np.all((x[bg] >= 0) & (x[bg] < 1))
    for a in range(3):
        assert ks_one(x[bg, a], lambda t: t) < 1.95 / math.sqrt(nbg)
    sizes = prm["sizes"]
    assert sizes.sum() == n - nbg and np.all((prm["radii"] >= 0.01) & (prm["radii"] <= 0.1))
    assert np.all((prm["centres"] >= 0) & (prm["centres"] < 1))
    cap = mass(10.0)
    qc = q_cdf()
    o = 0
    for k in range(8):
        m = int(sizes[k])
        xs, vs = x[o:o + m], v[o:o + m]
        r = np.linalg.norm(xs - prm["centres"][k], axis=1) / prm["radii"][k]
        assert ks_one(r, lambda t: mass(t) / cap) < 1.95 / math.sqrt(m)
        scale = math.sqrt((m / n) / prm["radii"][k])
        assert np.allclose(vs.mean(axis=0), prm["bulk"][k], atol=5 * scale / math.sqrt(m))
        q = np.linalg.norm(vs - prm["bulk"][k], axis=1) / (scale * math.sqrt(2.0) * (r * r + 1) ** -0.25)
        assert ks_one(q, qc) < 1.95 / math.sqrt(m)
        o += m


def test_batch_systems_on_the_device():
    """gb_batch_init_plummer: each system a Plummer sphere of total mass 1
    scaled to its radius R_k in [0.5, 2]: radii / R_k follow the capped
    Plummer profile and speed fractions the distribution function's q law (KS
    over all systems pooled), and the largest systems are near virial
    equilibrium (2K / |W| within 0.1 of 1, potential from the FMM)."""
    import vipp_gb300
    rng = np.random.default_rng(3)
    sizes = np.rint(np.exp(rng.uniform(math.log(1024), math.log(16384), 24))).astype(np.int64)
    with vipp_gb300.Batch(sizes, p=6, s=32, eps=0.01, masses=1.0 / sizes, precision="fp64") as b:
        radii = b.init_plummer(seed=3)
        x, v = b.download()
        assert np.all((radii >= 0.5) & (radii <= 2.0))
        off = np.concatenate([[0], np.cumsum(sizes)])
        rs, qs = [], []
        for k in range(len(sizes)):
            xs, vs = x[off[k]:off[k + 1]], v[off[k]:off[k + 1]]
            r = np.linalg.norm(xs, axis=1) / radii[k]
            rs.append(r)
            qs.append(np.linalg.norm(vs, axis=1) * math.sqrt(radii[k]) / (math.sqrt(2.0) * (r * r + 1) ** -0.25))
        r, q = np.concatenate(rs), np.concatenate(qs)
        assert ks_one(r, lambda t: mass(t) / mass(10.0)) < 1.95 / math.sqrt(len(r))
        assert ks_one(q, q_cdf()) < 1.95 / math.sqrt(len(q))
        for k in np.argsort(sizes)[-3:]:
            cons = b.system_conserved(int(k))
            assert abs(2 * cons["kinetic"] / abs(cons["potential"]) - 1) < 0.1
