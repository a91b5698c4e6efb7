"""Wisdom text format and bookkeeping (host only, no GPU needed)."""
import ctypes

import pfft_gb300 as pg

HDR = "pfft_gb300-wisdom 2\n"
HDR1 = "pfft_gb300-wisdom 1\n"


def test_forget_export_import(pfft_lib):
    L = pg.lib()
    L.pfft_gb300_forget_wisdom()
    assert L.pfft_gb300_wisdom_entries() == 0
    assert pg.export_wisdom() == HDR
    w = HDR + "a2.m0.s-1.N512.key 0 8 0 0 1\na0.m1.s-1.N96.key 1 0 2 16 0\n"
    assert L.pfft_gb300_import_wisdom_from_string(w.encode()) == 1
    assert L.pfft_gb300_wisdom_entries() == 2
    out = pg.export_wisdom()
    assert out.startswith(HDR) and "a0.m1.s-1.N96.key 1 0 2 16 0" in out and "a2.m0.s-1.N512.key 0 8 0 0 1" in out
    # the first format (no staged field) is still read, with staged = 0
    assert L.pfft_gb300_import_wisdom_from_string((HDR1 + "a1.m0.s1.N32.key 0 0 0 0\n").encode()) == 1
    assert "a1.m0.s1.N32.key 0 0 0 0 0" in pg.export_wisdom()
    L.pfft_gb300_forget_wisdom()
    assert L.pfft_gb300_wisdom_entries() == 0


def test_import_rejects_malformed(pfft_lib):
    L = pg.lib()
    L.pfft_gb300_forget_wisdom()
    for bad in ["", "not wisdom\n", HDR + "key 0 0 0 0\n", HDR + "key 2 0 0 0 0\n", HDR + "key 1 0 7 4 0\n",
                HDR + "key x 0 0 0 0\n", HDR + "key 0 0 0 0 3\n", HDR1 + "key 0 0 0\n"]:
        assert L.pfft_gb300_import_wisdom_from_string(bad.encode()) == 0, bad
    assert L.pfft_gb300_wisdom_entries() == 0  # nothing half-imported


def test_file_roundtrip(pfft_lib, tmp_path):
    L = pg.lib()
    L.pfft_gb300_forget_wisdom()
    w = HDR + "a1.m0.s1.N64.key 1 0 1 8 2\n"
    assert L.pfft_gb300_import_wisdom_from_string(w.encode()) == 1
    f = str(tmp_path / "w.txt")
    assert L.pfft_gb300_export_wisdom_to_filename(f.encode()) == 1
    L.pfft_gb300_forget_wisdom()
    assert L.pfft_gb300_import_wisdom_from_filename(f.encode()) == 1
    assert pg.export_wisdom() == w
    assert L.pfft_gb300_import_wisdom_from_filename(str(tmp_path / "missing").encode()) == 0
    L.pfft_gb300_forget_wisdom()
