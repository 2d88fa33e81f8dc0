"""The synthetic workload generators (vipp_gb300.workloads; host, numpy):
determinism, layout, and the analytic properties of the clustered stress
workload's components (CPU only)."""
import math

import numpy as np

from vipp_gb300.workloads import clustered, plummer

# Plummer sphere with radii capped at 10 a: half-mass radius r_h solves
# r^3 / (1 + r^2)^1.5 = f(10) / 2 (r in units of a) ...
HALF_MASS_CAPPED = 1.2874854
# ... and the mean squared speed is 3 pi / 32 G M / a uncapped (virial
# theorem); the cap removes some of the slowest outer particles.
MEAN_V2 = 3 * math.pi / 32


def test_plummer_deterministic():
    a = plummer(4096, 2)
    b = plummer(4096, 2)
    c = plummer(4096, 3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])
    assert np.all(np.linalg.norm(a[0], axis=1) <= 10.0)
    assert a[0].flags.c_contiguous and a[0].shape == (4096, 3)


def test_clustered_layout_and_components():
    n = 1 << 18
    x, v, info = clustered(n, 4)
    x2, v2, _ = clustered(n, 4)
    assert np.array_equal(x, x2) and np.array_equal(v, v2)
    sizes, nbg = info["sizes"], info["background"]
    assert nbg == round(0.05 * n) and int(sizes.sum()) + nbg == n
    assert sizes.max() - sizes.min() <= 1
    assert np.all((info["radii"] >= 0.01) & (info["radii"] <= 0.1))
    assert np.all((info["centres"] >= 0) & (info["centres"] < 1))
    bg = slice(n - nbg, n)
    assert np.all((x[bg] >= 0) & (x[bg] < 1)) and np.all(v[bg] == 0)
    o = 0
    for k in range(len(sizes)):
        m, a = int(sizes[k]), info["radii"][k]
        xc = x[o:o + m] - info["centres"][k]
        vc = v[o:o + m] - info["bulk"][k]
        r = np.linalg.norm(xc, axis=1)
        assert r.max() <= 10 * a * (1 + 1e-12)
        assert abs(np.median(r) / a / HALF_MASS_CAPPED - 1) < 0.03
        v2 = np.mean(np.sum(vc * vc, axis=1)) / ((m / n) / a)
        assert abs(v2 / MEAN_V2 - 1) < 0.04
        assert np.all(np.abs(vc.mean(axis=0)) < 0.02 * math.sqrt((m / n) / a))
        o += m
