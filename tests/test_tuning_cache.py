"""The autotuner's cache file and its reader in the library
(gb_tuning_lookup, vipp_gb300/autotune.py): format, bucket selection,
validation. No GPU needed: the lookup only reads the file."""
import pytest

import vipp_gb300
from vipp_gb300 import autotune


def entry(log2n, p=8, precision=1, mode=0, bf16=1, **t):
    key = {"p": p, "precision": precision, "mode": mode, "m2l_bf16": bf16, "log2n": log2n}
    tun = dict(vipp_gb300.TUNING_DEFAULT)
    tun.update(t)
    return key, tun


def test_lookup_selects_the_bucket_and_configuration(tmp_path):
    vipp_gb300.load()
    path = str(tmp_path / "tune.txt")
    autotune.write_cache(path, [entry(22, p2p_blocks=6, p2p_slice=4096), entry(20, p2p_blocks_conc=4),
                                entry(22, precision=0, m2l_ctas_pct=50), entry(16, p=6, serial=1),
                                entry(14, p=10, mode=1, bf16=0, leaf_s=80)])
    got = vipp_gb300.tuning_lookup(path, 1 << 22, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)
    assert got["p2p_blocks"] == 6 and got["p2p_slice"] == 4096 and got["m2l_ctas_pct"] == 100
    # bucket floor(log2 n): 5,000,000 is in bucket 22, 2^20 + 1 in bucket 20
    assert vipp_gb300.tuning_lookup(path, 5_000_000, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)["p2p_blocks"] == 6
    assert vipp_gb300.tuning_lookup(path, (1 << 20) + 1, 8, "mixed", "ref",
                                    vipp_gb300.FLAG_M2L_BF16)["p2p_blocks_conc"] == 4
    assert vipp_gb300.tuning_lookup(path, 1 << 22, 8, "fp64", "ref", vipp_gb300.FLAG_M2L_BF16)["m2l_ctas_pct"] == 50
    assert vipp_gb300.tuning_lookup(path, 70000, 6, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)["serial"] == 1
    assert vipp_gb300.tuning_lookup(path, 20000, 10, "mixed", "accurate", 0)["leaf_s"] == 80
    # no entry: other split, other order, other bucket
    assert vipp_gb300.tuning_lookup(path, 1 << 22, 8, "mixed", "ref", 0) is None
    assert vipp_gb300.tuning_lookup(path, 1 << 22, 7, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16) is None
    assert vipp_gb300.tuning_lookup(path, 1 << 21, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16) is None


def test_last_entry_wins_and_comments(tmp_path):
    vipp_gb300.load()
    path = tmp_path / "tune.txt"
    k, t = entry(22, p2p_blocks=4)
    k2, t2 = entry(22, p2p_blocks=7)
    path.write_text("# header\n\n" + autotune.cache_line(k, t, "first") + "\n" + autotune.cache_line(k2, t2) + "  # later\n")
    assert vipp_gb300.tuning_lookup(str(path), 1 << 22, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)["p2p_blocks"] == 7
    assert autotune.read_cache(str(path)) == [(k, t), (k2, t2)]


@pytest.mark.parametrize("line", ["p=8 precision=1 mode=0 m2l_bf16=1 log2n=22 p2p_slice=100",  # out of range
                                  "p=8 precision=1 mode=0 m2l_bf16=1 log2n=22 bogus=3",         # unknown key
                                  "p=8 precision=1 mode=0 m2l_bf16=1 p2p_blocks=4",            # no bucket
                                  "p=8 precision=1 mode=0 m2l_bf16=1 log2n=22 p2p_blocks=x",   # not a number
                                  "p=8 precision=1 mode=0 m2l_bf16=1 log2n=22 p2p_occupancy=7"])  # no such build
def test_malformed_entries_are_rejected(tmp_path, line):
    vipp_gb300.load()
    path = tmp_path / "tune.txt"
    path.write_text(line + "\n")
    with pytest.raises(vipp_gb300.GB300Error) as ei:
        vipp_gb300.tuning_lookup(str(path), 1 << 22, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)
    assert ei.value.code == vipp_gb300.GB_ERR_INVALID


def test_missing_file_is_an_error(tmp_path):
    vipp_gb300.load()
    with pytest.raises(vipp_gb300.GB300Error):
        vipp_gb300.tuning_lookup(str(tmp_path / "none.txt"), 1000, 4)


def test_shipped_cache_parses():
    """The library's GB300 cache (vipp_gb300/tuning_gb300.txt, which bench.py
    applies by default) is well formed and holds the headline buckets."""
    import os
    vipp_gb300.load()
    path = os.path.join(os.path.dirname(vipp_gb300.__file__), "tuning_gb300.txt")
    entries = autotune.read_cache(path)
    assert len(entries) >= 3
    acc = vipp_gb300.tuning_lookup(path, 1 << 22, 10, "mixed", "accurate", 0)
    assert acc is not None and acc["leaf_s"] >= 64
    ref = vipp_gb300.tuning_lookup(path, 1 << 22, 8, "mixed", "ref", vipp_gb300.FLAG_M2L_BF16)
    assert ref is not None and ref["p2p_blocks_conc"] < ref["p2p_blocks"]  # P2P beside the M2L on a share of the SMs
    assert ref["p2p_occupancy"] == 6 and acc["p2p_occupancy"] == 8
