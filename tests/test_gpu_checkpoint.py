"""Checkpoint save and load on the GPU: a run restarted from a checkpoint
continues bit-identically to the run that wrote it (context, forest batch and
contexts batch, and across the two batch forms); the step count and time come
back; a checkpoint with another configuration, other systems or a corrupt body
is refused and leaves the state as it was."""
import numpy as np
import pytest

import vipp_gb300

pytestmark = pytest.mark.gpu

DT = 1e-3


def solver(**kw):
    cfg = dict(p=6, s=32, eps=0.01, precision="mixed", flags=vipp_gb300.FLAG_M2L_BF16)
    cfg.update(kw)
    return vipp_gb300.Solver(**cfg)


@pytest.mark.parametrize("precision,flags", [("mixed", vipp_gb300.FLAG_M2L_BF16), ("fp64", 0)])
def test_context_restart_is_bit_identical(tmp_path, precision, flags):
    path = str(tmp_path / "ctx.ckpt")
    with solver(precision=precision, flags=flags) as a:
        a.init_plummer(20000, seed=5)
        for _ in range(3):
            a.solve(DT)
        a.save_checkpoint(path, t=3 * DT)
        assert a.stats()["steps"] == 3
        x3, v3 = a.postprocess()
        a.solve(DT)
        a.solve(DT)
        xa, va = a.postprocess()
    got = vipp_gb300.checkpoint_read(path)
    assert got["steps"] == 3 and got["t"] == 3 * DT and got["nsys"] == 1
    assert np.array_equal(got["x"], x3) and np.array_equal(got["v"], v3)
    with solver(precision=precision, flags=flags) as b:
        assert b.load_checkpoint(path) == 3 * DT
        assert b.stats()["steps"] == 3
        b.solve(DT)
        b.solve(DT)
        xb, vb = b.postprocess()
        assert b.stats()["steps"] == 5
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_configuration_is_checked_and_a_refused_load_keeps_the_state(tmp_path):
    path = str(tmp_path / "c.ckpt")
    with solver() as a:
        a.init_plummer(4000, seed=2)
        a.solve(DT)
        a.save_checkpoint(path)
    for kw, word in ((dict(p=4), "p 6"), (dict(eps=0.02), "eps"), (dict(flags=0), "flags"),
                     (dict(precision="fp64"), "precision")):
        with solver(**kw) as b:
            b.init_plummer(1000, seed=9)
            x0, v0 = b.postprocess()
            t0 = b.tuning()
            with pytest.raises(vipp_gb300.GB300Error) as ei:
                b.load_checkpoint(path)
            assert ei.value.code == vipp_gb300.GB_ERR_INVALID and word in str(ei.value), str(ei.value)
            x1, v1 = b.postprocess()
            assert np.array_equal(x0, x1) and np.array_equal(v0, v1) and b.tuning() == t0
    with solver(p=4) as b:  # any_config: the state loads into another configuration
        b.load_checkpoint(path, any_config=True)
        assert b.n == 4000 and b.stats()["steps"] == 1
    raw = bytearray(open(path, "rb").read())
    raw[-40] ^= 1
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(raw)
    with solver() as b:
        b.init_plummer(1000, seed=9)
        x0, _ = b.postprocess()
        with pytest.raises(vipp_gb300.GB300Error, match="check word"):
            b.load_checkpoint(bad)
        assert np.array_equal(b.postprocess()[0], x0)


def test_save_before_upload_is_a_state_error(tmp_path):
    with solver() as a:
        with pytest.raises(vipp_gb300.GB300Error) as ei:
            a.save_checkpoint(str(tmp_path / "x.ckpt"))
        assert ei.value.code == vipp_gb300.GB_ERR_STATE


SIZES = [3000, 0, 5000, 1, 1200]


def batch(form, **kw):
    flags = vipp_gb300.FLAG_M2L_BF16 | (vipp_gb300.FLAG_BATCH_CONTEXTS if form == "contexts" else 0)
    masses = 1.0 / np.maximum(np.asarray(SIZES), 1)
    cfg = dict(p=4, s=16, eps=0.01, masses=masses, precision="mixed", flags=flags)
    cfg.update(kw)
    return vipp_gb300.Batch(SIZES, **cfg)


@pytest.mark.parametrize("writer,reader", [("forest", "forest"), ("contexts", "contexts"), ("forest", "contexts")])
def test_batch_restart_is_bit_identical(tmp_path, writer, reader):
    path = str(tmp_path / "b.ckpt")
    with batch(writer) as a:
        a.init_plummer(seed=4)
        a.step(DT)
        a.step(DT)
        a.save_checkpoint(path, t=2 * DT)
        a.step(DT)
        xa, va = a.download()
        assert a.stats()["steps"] == 3
    got = vipp_gb300.checkpoint_read(path, arrays=False)
    assert got["nsys"] == len(SIZES) and got["n"] == sum(SIZES) and got["steps"] == 2
    with batch(reader) as b:
        assert b.load_checkpoint(path) == 2 * DT
        b.step(DT)
        xb, vb = b.download()
        assert b.stats()["steps"] == 3
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_batch_checkpoint_must_match_the_systems(tmp_path):
    path = str(tmp_path / "b.ckpt")
    with batch("forest") as a:
        a.init_plummer(seed=4)
        a.save_checkpoint(path)
        lib = vipp_gb300.load()  # the forest context itself saves through its batch only
        assert lib.gb_checkpoint_save(lib.gb_batch_forest(a.h), str(tmp_path / "f.ckpt").encode(), 0.0) == 1
    with solver(p=4, s=16) as s:
        with pytest.raises(vipp_gb300.GB300Error, match="5 systems"):
            s.load_checkpoint(path)
    other = list(SIZES)
    other[0], other[2] = other[2], other[0]
    with vipp_gb300.Batch(other, p=4, s=16, eps=0.01, masses=1.0 / np.maximum(np.asarray(other), 1),
                          precision="mixed", flags=vipp_gb300.FLAG_M2L_BF16) as b:
        with pytest.raises(vipp_gb300.GB300Error, match="segment offsets"):
            b.load_checkpoint(path)
    with batch("forest", masses=np.full(len(SIZES), 0.5)) as b:
        with pytest.raises(vipp_gb300.GB300Error, match="mass of system 0"):
            b.load_checkpoint(path)
        b.load_checkpoint(path, any_config=True)
