"""Tuning knobs (gb_set_tuning) and the tuning cache applied at upload
(VIPP_GB_TUNE_FILE) on the GPU.

  * launch shapes (P2P blocks per SM alone and beside the far field, M2L CTAs,
    serial near field): bit-identical accelerations and RK4 steps;
  * P2P slice length: only the FP32 summation order of long near-field lists
    changes: within the mixed tolerance (RMS <= 2e-6, max <= 1e-4) of the
    default;
  * leaf_s (accurate mode only): another tree, and still <= 1e-5 RMS from the
    FP64 direct sum at p = 10; the reference mode ignores it.
"""
import math

import numpy as np
import pytest

import oracle as O
from treecmp import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plummer64k():
    from vipp_gb300.workloads import plummer
    return plummer(1 << 16, 2)


def run(x, v, tune=None, **kw):
    import vipp_gb300
    n = x.shape[0]
    with vipp_gb300.Solver(m=1.0 / n, **kw) as s:
        if tune:
            s.set_tuning(**tune)
        s.preprocess(x, v)
        a = s.accel()
        s.solve(5e-4)
        xs, vs = s.postprocess()
        st = s.stats()
        t = s.tuning()
    return a, xs, vs, st, t


CFG = dict(p=8, s=64, eps=0.005, precision="mixed")


@pytest.mark.parametrize("tune", [{"p2p_blocks": 4}, {"p2p_blocks_conc": 0}, {"p2p_blocks_conc": 3, "m2l_ctas_pct": 50},
                                  {"serial": 1}, {"m2l_ctas_pct": 10}, {"p2p_occupancy": 6},
                                  {"p2p_occupancy": 6, "p2p_blocks_conc": 2}])
def test_launch_shapes_are_bit_identical(plummer64k, tune):
    import vipp_gb300
    x, v = plummer64k
    a0, x0, v0, _, _ = run(x, v, flags=vipp_gb300.FLAG_M2L_BF16, **CFG)
    a1, x1, v1, _, t = run(x, v, tune, flags=vipp_gb300.FLAG_M2L_BF16, **CFG)
    assert all(t[k] == val for k, val in tune.items())
    assert np.array_equal(a0, a1) and np.array_equal(x0, x1) and np.array_equal(v0, v1)


@pytest.mark.parametrize("slice_", [1024, 2048, 32768])
def test_slice_length_changes_only_rounding(plummer64k, slice_):
    x, v = plummer64k
    a0, *_ = run(x, v, **CFG)
    a1, *_ = run(x, v, {"p2p_slice": slice_}, **CFG)
    e = rel_err(a1, a0)
    assert math.sqrt(np.mean(e * e)) <= 2e-6 and np.max(e) <= 1e-4


def test_leaf_s_in_accurate_mode_only(plummer64k):
    x, v = plummer64k
    x, v = x[:16384].copy(), v[:16384].copy()
    n = x.shape[0]
    ad = O.direct_accel(x, 1.0, 1.0 / n, 0.005)
    a0, _, _, st0, _ = run(x, v, p=10, s=64, eps=0.005, precision="mixed", mode="accurate")
    a1, _, _, st1, _ = run(x, v, {"leaf_s": 96}, p=10, s=64, eps=0.005, precision="mixed", mode="accurate")
    assert st1["ncells"] < st0["ncells"]
    for a in (a0, a1):
        e = rel_err(a, ad)
        assert math.sqrt(np.mean(e * e)) <= 1e-5
    ar, _, _, str_, _ = run(x, v, {"leaf_s": 96}, p=10, s=64, eps=0.005, precision="mixed")
    assert str_["ncells"] == st0["ncells"]  # the reference mode keeps the config's s


def test_cache_is_applied_at_upload(plummer64k, tmp_path, monkeypatch):
    import vipp_gb300
    from vipp_gb300 import autotune
    x, v = plummer64k
    n = x.shape[0]
    key = autotune.bucket_key(n, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)
    tun = dict(vipp_gb300.TUNING_DEFAULT, p2p_blocks=5, p2p_blocks_conc=2, m2l_ctas_pct=60)
    path = str(tmp_path / "tune.txt")
    autotune.write_cache(path, [(key, tun)])
    monkeypatch.setenv("VIPP_GB_TUNE_FILE", path)
    a1, x1, v1, _, t = run(x, v, flags=vipp_gb300.FLAG_M2L_BF16, **CFG)
    assert t == tun
    monkeypatch.delenv("VIPP_GB_TUNE_FILE")
    a0, x0, v0, _, t0 = run(x, v, flags=vipp_gb300.FLAG_M2L_BF16, **CFG)
    assert t0 == vipp_gb300.TUNING_DEFAULT
    assert np.array_equal(a0, a1) and np.array_equal(x0, x1)


def test_tuner_picks_a_measured_candidate(plummer64k):
    """A short coordinate-descent run on 65,536 particles returns a valid
    tuning no slower than the defaults it also measured."""
    import vipp_gb300
    from vipp_gb300 import autotune
    x, v = plummer64k
    r = autotune.tune(x, v, p=6, s=64, eps=0.005, m=1.0 / x.shape[0], flags=vipp_gb300.FLAG_M2L_BF16, steps=1, sweeps=1)
    assert set(r["tuning"]) == set(vipp_gb300.TUNING_FIELDS) and r["trials"] >= 10
    assert r["tuned_s"] <= r["default_s"] * 1.05
