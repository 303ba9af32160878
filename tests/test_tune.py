"""The per-size-class tuning table of the plain primitives (host side, no
GPU): set / get with nearest-class lookup, save / load round trip, malformed
lines, and the committed table parses."""
import ctypes
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
TABLE = ROOT / "efficient-dpp_gb300" / "tuning" / "plain_gb300.tsv"


@pytest.fixture
def lib(edpp):
    L = edpp.lib()
    yield L
    L.edpp_tune_load(None)  # back to the committed table for later tests


def test_variant_counts(lib, edpp):
    assert lib.edpp_tune_variants(edpp.TUNE_SCAN_LOOKBACK) == 4
    assert lib.edpp_tune_variants(edpp.TUNE_SCAN_RTS) == 5
    assert lib.edpp_tune_variants(edpp.TUNE_GATHER) == 2
    assert lib.edpp_tune_variants(7) == 0


def test_set_get_nearest_class(lib, edpp):
    lib.edpp_tune_clear()
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, 1 << 24) == (0, False)  # default
    edpp.tune_set(edpp.TUNE_SCAN_LOOKBACK, 4, 20, 1)
    edpp.tune_set(edpp.TUNE_SCAN_LOOKBACK, 4, 28, 2)
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, 1 << 20) == (1, True)
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, (1 << 21) + 5) == (1, True)  # class 21 -> 20
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, 1 << 24) == (2, True)  # tie -> larger
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, 1 << 30) == (2, True)
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 8, 1 << 20) == (0, False)  # other element size
    assert edpp.tune_get(edpp.TUNE_GATHER, 4, 1 << 20) == (0, False)  # other primitive
    # out-of-range arguments
    assert lib.edpp_tune_set(edpp.TUNE_SCAN_LOOKBACK, 4, 20, 4, ctypes.c_float(0)) == edpp.EDPP_EINVAL
    assert lib.edpp_tune_set(edpp.TUNE_SCAN_LOOKBACK, 2, 20, 0, ctypes.c_float(0)) == edpp.EDPP_EINVAL
    assert lib.edpp_tune_set(9, 4, 20, 0, ctypes.c_float(0)) == edpp.EDPP_EINVAL


def test_save_load_round_trip(lib, edpp, tmp_path):
    lib.edpp_tune_clear()
    edpp.tune_set(edpp.TUNE_GATHER, 4, 25, 1, 0.49)
    edpp.tune_set(edpp.TUNE_SCAN_RTS, 8, 29, 2, 4.0)
    edpp.tune_set(edpp.TUNE_SCAN_LOOKBACK, 4, 24, 1, 0.05)
    p = tmp_path / "t.tsv"
    edpp.tune_save(p)
    lines = [l for l in p.read_text().splitlines() if l and not l.startswith("#")]
    assert lines == ["scan_lookback 4 24 1 0.0500", "scan_rts 8 29 2 4.0000",
                     "gather 4 25 1 0.4900"]
    lib.edpp_tune_clear()
    assert edpp.tune_load(p) == edpp.EDPP_OK
    assert edpp.tune_get(edpp.TUNE_GATHER, 4, 1 << 25) == (1, True)
    assert edpp.tune_get(edpp.TUNE_SCAN_RTS, 8, 1 << 29) == (2, True)


def test_malformed_lines_are_skipped(lib, edpp, tmp_path):
    p = tmp_path / "bad.tsv"
    p.write_text("# comment\n\nscan_lookback 4 24 1 0.05\nscan_lookback 4 25 7 0.1\n"
                 "nosuch 4 24 0 0\ngather 3 24 0 0\ngather 4 26 1  # trailing comment\n")
    assert edpp.tune_load(p) == edpp.EDPP_EINVAL
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, 1 << 24) == (1, True)
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, 1 << 25) == (1, True)  # bad line skipped
    assert edpp.tune_get(edpp.TUNE_GATHER, 4, 1 << 26) == (1, True)
    assert edpp.tune_load(tmp_path / "missing.tsv") == edpp.EDPP_OK  # empty table
    assert edpp.tune_get(edpp.TUNE_GATHER, 4, 1 << 26) == (0, False)


def test_committed_table_parses(lib, edpp):
    if not TABLE.exists():
        pytest.skip("no committed tuning table")
    assert edpp.tune_load(TABLE) == edpp.EDPP_OK
    assert edpp.tune_load(None) == edpp.EDPP_OK  # the default path is the same file
    rows = [l.split() for l in TABLE.read_text().splitlines() if l and not l.startswith("#")]
    assert rows
    for name, elem, cls, variant, _ms in rows:
        prim = {v: k for k, v in edpp.TUNE_NAMES.items()}[name]
        assert edpp.tune_get(prim, int(elem), 1 << int(cls)) == (int(variant), True)


def test_autotune_rejects_bad_arguments(lib, edpp):
    fake = ctypes.c_void_p(256)
    v = ctypes.c_int()
    ms = ctypes.c_float()
    A = lib.edpp_autotune_plain
    assert A(9, fake, fake, None, 100, 4, fake, 1 << 20, None, 1, None, 0,
             ctypes.byref(v), ctypes.byref(ms), None) == edpp.EDPP_EINVAL
    assert A(edpp.TUNE_GATHER, fake, fake, None, 100, 4, fake, 1 << 20, None, 1, None, 0,
             ctypes.byref(v), ctypes.byref(ms), None) == edpp.EDPP_EINVAL  # gather needs loc
    assert A(edpp.TUNE_SCAN_LOOKBACK, fake, fake, None, 100, 2, fake, 1 << 20, None, 1, None, 0,
             ctypes.byref(v), ctypes.byref(ms), None) == edpp.EDPP_EINVAL
    assert A(edpp.TUNE_SCAN_LOOKBACK, fake, fake, None, 0, 4, fake, 1 << 20, None, 1, None, 0,
             ctypes.byref(v), ctypes.byref(ms), None) == edpp.EDPP_EINVAL
