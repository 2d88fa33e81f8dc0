"""Checkpoint files (gb_checkpoint_write / gb_checkpoint_read): the documented
byte layout, the round trip, the check word and the rejection of malformed,
truncated and corrupt files and bad arguments. Host code only: no GPU."""
import ctypes
import os
import struct

import numpy as np
import pytest

import vipp_gb300

FNV_BASIS, FNV_PRIME, MASK = 0xcbf29ce484222325, 0x100000001b3, (1 << 64) - 1


def fnv_words(data: bytes) -> int:
    """FNV-1a over 64-bit little-endian words, one word per round (the check word)."""
    h = FNV_BASIS
    for (w,) in struct.iter_unpack("<Q", data):
        h = ((h ^ w) * FNV_PRIME) & MASK
    return h


def sample(n=50, nsys=3, seed=1):
    rng = np.random.default_rng(seed)
    x, v = rng.normal(size=(n, 3)), rng.normal(size=(n, 3)) * 1e-3
    cuts = np.sort(rng.integers(0, n + 1, nsys - 1))
    seg = np.concatenate([[0], cuts, [n]]).astype(np.uint64)
    masses = rng.uniform(0.5, 2.0, nsys) / n
    return x, v, seg, masses


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not os.path.exists(vipp_gb300.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return vipp_gb300.load()


def test_round_trip_is_bit_exact(tmp_path):
    x, v, seg, masses = sample()
    x[3, 1] = -0.0
    x[4, 2] = 5e-324  # subnormal
    path = str(tmp_path / "state.ckpt")
    vipp_gb300.checkpoint_write(path, x, v, p=8, s=64, eps=0.005, G=1.0, m=0.25, precision="mixed",
                                flags=vipp_gb300.FLAG_M2L_BF16, mode="ref", seg=seg, masses=masses, steps=17,
                                t=0.0085, leaf_s=64)
    got = vipp_gb300.checkpoint_read(path)
    assert (got["n"], got["nsys"], got["steps"], got["t"], got["leaf_s"]) == (50, 3, 17, 0.0085, 64)
    assert got["config"] == {"p": 8, "s": 64, "eps": 0.005, "G": 1.0, "m": 0.25, "precision": 1,
                             "flags": vipp_gb300.FLAG_M2L_BF16, "mode": 0}
    for k, a in (("x", x), ("v", v), ("seg", seg), ("masses", masses)):
        assert got[k].tobytes() == np.ascontiguousarray(a).tobytes(), k
    assert not os.path.exists(path + ".tmp")


def test_byte_layout_matches_the_header_documentation(tmp_path):
    x, v, seg, masses = sample(n=7, nsys=2, seed=3)
    path = str(tmp_path / "a.ckpt")
    vipp_gb300.checkpoint_write(path, x, v, p=6, s=32, eps=0.01, G=2.0, m=0.5, precision="fp64", flags=3, mode="accurate",
                                seg=seg, masses=masses, steps=4, t=1.5, leaf_s=80)
    raw = open(path, "rb").read()
    n, ns = 7, 2
    assert len(raw) == 128 + 8 * ((ns + 1) + ns + 6 * n) + 8
    assert raw[:8] == b"VIPPGBCK"
    assert struct.unpack_from("<IIQQqd", raw, 8) == (1, 128, n, ns, 4, 1.5)
    assert struct.unpack_from("<6i", raw, 48) == (6, 32, 0, 1, 3, 80)
    assert struct.unpack_from("<3d", raw, 72) == (0.01, 2.0, 0.5)
    assert raw[96:128] == bytes(32)
    o = 128
    assert np.array_equal(np.frombuffer(raw, "<u8", ns + 1, o), seg)
    o += 8 * (ns + 1)
    assert np.array_equal(np.frombuffer(raw, "<f8", ns, o), masses)
    o += 8 * ns
    assert np.array_equal(np.frombuffer(raw, "<f8", 3 * n, o).reshape(n, 3), x)
    o += 24 * n
    assert np.array_equal(np.frombuffer(raw, "<f8", 3 * n, o).reshape(n, 3), v)
    o += 24 * n
    assert struct.unpack_from("<Q", raw, o)[0] == fnv_words(raw[:o])


def test_one_system_defaults_and_empty_state(tmp_path):
    path = str(tmp_path / "one.ckpt")
    x, v, _, _ = sample(n=5)
    vipp_gb300.checkpoint_write(path, x, v, m=0.2)
    got = vipp_gb300.checkpoint_read(path)
    assert got["nsys"] == 1 and list(got["seg"]) == [0, 5] and list(got["masses"]) == [0.2]
    empty = str(tmp_path / "empty.ckpt")
    vipp_gb300.checkpoint_write(empty, np.zeros((0, 3)), np.zeros((0, 3)))
    got = vipp_gb300.checkpoint_read(empty)
    assert got["n"] == 0 and got["x"].shape == (0, 3) and list(got["seg"]) == [0, 0]


def test_overwrite_replaces_the_file(tmp_path):
    path = str(tmp_path / "s.ckpt")
    x, v, _, _ = sample(n=9)
    vipp_gb300.checkpoint_write(path, x, v, steps=1)
    vipp_gb300.checkpoint_write(path, x[:4], v[:4], steps=2)
    got = vipp_gb300.checkpoint_read(path)
    assert got["n"] == 4 and got["steps"] == 2 and os.listdir(tmp_path) == ["s.ckpt"]


def expect_invalid(fn, *words):
    with pytest.raises(vipp_gb300.GB300Error) as ei:
        fn()
    assert ei.value.code == vipp_gb300.GB_ERR_INVALID
    for w in words:
        assert w in str(ei.value), (w, str(ei.value))


def test_corruption_is_detected_by_the_check_word(tmp_path):
    path = str(tmp_path / "c.ckpt")
    x, v, seg, masses = sample()
    vipp_gb300.checkpoint_write(path, x, v, seg=seg, masses=masses)
    raw = bytearray(open(path, "rb").read())
    raw[128 + 8 * 7 + 100] ^= 0x10  # a bit of the positions
    open(path, "wb").write(raw)
    assert vipp_gb300.checkpoint_read(path, arrays=False)["n"] == 50  # the header alone is intact
    expect_invalid(lambda: vipp_gb300.checkpoint_read(path), "check word")


def test_malformed_files_are_rejected(tmp_path):
    x, v, seg, masses = sample()
    good = str(tmp_path / "g.ckpt")
    vipp_gb300.checkpoint_write(good, x, v, seg=seg, masses=masses)
    raw = open(good, "rb").read()

    def variant(name, data):
        p = str(tmp_path / name)
        open(p, "wb").write(data)
        return p

    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("t.ckpt", raw[:-9])), "bytes")
    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("l.ckpt", raw + bytes(8))), "bytes")
    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("h.ckpt", raw[:60])), "header")
    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("m.ckpt", b"VIPPGBCX" + raw[8:])), "magic")
    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("v.ckpt", raw[:8] + struct.pack("<I", 2) + raw[12:])),
                   "version 2")
    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("z.ckpt", raw[:24] + struct.pack("<Q", 0) + raw[32:])),
                   "system count")
    expect_invalid(lambda: vipp_gb300.checkpoint_read(str(tmp_path / "none.ckpt")), "cannot open")
    # segment offsets that decrease, with a check word that matches them
    bad = bytearray(raw[:-8])
    struct.pack_into("<Q", bad, 128 + 8, 60)
    bad += struct.pack("<Q", fnv_words(bytes(bad)))
    expect_invalid(lambda: vipp_gb300.checkpoint_read(variant("s.ckpt", bytes(bad))), "segment")


def test_bad_write_arguments_are_rejected(tmp_path):
    x, v, _, _ = sample(n=10)
    p = str(tmp_path / "w.ckpt")
    expect_invalid(lambda: vipp_gb300.checkpoint_write(p, x, v, seg=[1, 10]), "from 0 to n")
    expect_invalid(lambda: vipp_gb300.checkpoint_write(p, x, v, seg=[0, 9]), "from 0 to n")
    expect_invalid(lambda: vipp_gb300.checkpoint_write(p, x, v, seg=[0, 6, 4, 10]), "decrease")
    expect_invalid(lambda: vipp_gb300.checkpoint_write(p, x, v, steps=-1), "step count")
    expect_invalid(lambda: vipp_gb300.checkpoint_write(str(tmp_path / "no" / "dir.ckpt"), x, v), "cannot open")
    assert not os.path.exists(p)
    lib = vipp_gb300.load()
    info = vipp_gb300.GbCheckpointInfo()
    info.n, info.nsys = 10, 2
    assert lib.gb_checkpoint_write(p.encode(), ctypes.byref(info), None, None, None, None) == vipp_gb300.GB_ERR_INVALID
    assert b"null" in lib.gb_last_error(None)
    info.n = 0
    assert lib.gb_checkpoint_write(p.encode(), ctypes.byref(info), None, None, None, None) == vipp_gb300.GB_ERR_INVALID
    assert b"segment offsets are needed" in lib.gb_last_error(None)
    assert lib.gb_checkpoint_write(None, ctypes.byref(info), None, None, None, None) == vipp_gb300.GB_ERR_INVALID


def test_read_capacities_are_checked(tmp_path):
    x, v, seg, masses = sample(n=20, nsys=4)
    p = str(tmp_path / "r.ckpt")
    vipp_gb300.checkpoint_write(p, x, v, seg=seg, masses=masses)
    lib = vipp_gb300.load()
    info = vipp_gb300.GbCheckpointInfo()
    xs, vs = np.zeros((20, 3)), np.zeros((20, 3))
    sg, ms = np.zeros(5, np.uint64), np.zeros(4)
    ptr = vipp_gb300._ptr
    assert lib.gb_checkpoint_read(p.encode(), ctypes.byref(info), None, None, 0, ptr(xs), ptr(vs), 19) == 1
    assert b"particle arrays too small" in lib.gb_last_error(None)
    assert lib.gb_checkpoint_read(p.encode(), ctypes.byref(info), ptr(sg), ptr(ms), 3, None, None, 0) == 1
    assert b"system arrays too small" in lib.gb_last_error(None)
    # only the positions: the body is still read through and checked
    assert lib.gb_checkpoint_read(p.encode(), ctypes.byref(info), None, None, 0, ptr(xs), None, 20) == 0
    assert np.array_equal(xs, x) and not vs.any()


def test_context_and_batch_calls_reject_null_handles():
    lib = vipp_gb300.load()
    INV = vipp_gb300.GB_ERR_INVALID
    t = ctypes.c_double()
    assert lib.gb_checkpoint_save(None, b"x", 0.0) == INV
    assert lib.gb_checkpoint_load(None, b"x", 0, ctypes.byref(t)) == INV
    assert lib.gb_batch_checkpoint_save(None, b"x", 0.0) == INV
    assert lib.gb_batch_checkpoint_load(None, b"x", 0, ctypes.byref(t)) == INV
