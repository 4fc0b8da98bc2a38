"""Table pipeline: reference tables extracted from source, synthetic k-tables
and the reference's 256 -> 140 g-point reduction (CPU only)."""
import os

import numpy as np

from brams_gb300.tables_io import read_tables

DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "brams_gb300", "data")
REF = read_tables(os.path.join(DATA, "lw_ref_tables.gblw"))
KT = read_tables(os.path.join(DATA, "lw_ktables.gblw"))
NG = [10, 12, 16, 14, 16, 8, 12, 8, 12, 6, 8, 8, 4, 2, 2, 2]


def test_reference_tables_shapes_and_anchor_values():
    assert REF["totplnk"].shape == (181, 16)
    assert REF["chi_mls"].shape == (7, 59)
    assert REF["absice3"].shape == (46, 16) and REF["absliq1"].shape == (58, 16)
    # values as written in the reference source
    assert REF["pref"][0] == 1.05363e+03 and REF["pref"][-1] == 9.65769e-03
    assert REF["preflog"][0] == 6.96 and REF["preflog"][12] == 4.56
    assert REF["totplnk"][0, 0] == 0.14783e-05
    assert list(REF["delwave"]) == [340., 150., 130., 70., 120., 160., 100., 100., 210., 90., 320., 280., 170., 130., 220., 650.]
    assert list(REF["nspa"]) == [1, 1, 9, 9, 9, 1, 9, 1, 9, 1, 1, 9, 9, 1, 9, 9]
    assert list(REF["nspb"]) == [1, 1, 5, 5, 5, 0, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0]
    assert REF["grav"] == 9.8066 and REF["abscld1"] == 0.0602410
    assert abs(REF["wt"].sum() - 1.0) < 1e-7  # the reference weights sum to 0.9999999791
    # preflog is ln(pref) to the 0.2-step grid the reference documents
    assert np.allclose(np.log(REF["pref"]), REF["preflog"], atol=2e-5)


def test_gpoint_maps_consistent():
    ngc, ngs, ngb, ngn = REF["ngc"], REF["ngs"], REF["ngb"], REF["ngn"]
    assert list(ngc) == NG and ngs[-1] == 140 and list(np.cumsum(ngc)) == list(ngs)
    for b in range(16):
        g0 = 0 if b == 0 else ngs[b - 1]
        assert np.all(ngb[g0:ngs[b]] == b + 1)
        assert ngn[g0:ngs[b]].sum() == 16  # every original g-point lands in one reduced interval


def test_ktable_shapes_match_reference_modules():
    assert KT["b03.ka"].shape == (9, 5, 13, 16)
    assert KT["b03.kb"].shape == (5, 5, 47, 16)
    assert KT["b01.ka"].shape == (5, 13, 10) and KT["b01.kb"].shape == (5, 47, 10)
    assert KT["b16.kb"].shape == (5, 47, 2)
    assert KT["b13.ka_mco"].shape == (9, 19, 4)
    assert KT["b08.ka_mo3"].shape == (19, 8)
    assert "b12.kb" not in KT and "b15.kb" not in KT and "b06.kb" not in KT
    total = sum(v.size for v in KT.values())
    assert total == 142866
    for k, v in KT.items():
        assert np.all(np.isfinite(v)) and np.all(v >= 0), k


def test_planck_fractions_sum_to_one():
    for b in range(1, 17):
        for nm in ("fracrefa", "fracrefb"):
            key = f"b{b:02d}.{nm}"
            if key in KT:
                f = KT[key]
                s = f.sum(axis=0)
                assert np.allclose(s, 1.0, atol=1e-12), key


def test_reduction_reproduces_committed_tables():
    """Regenerating the 16-point tables and applying cmbgb gives the committed file."""
    from brams_gb300.data.gen_ktables import make_original_tables, reduce_tables, rwgt_table

    orig = make_original_tables(REF)
    red = reduce_tables(orig, REF)
    assert set(red) == set(KT)
    for k in KT:
        assert np.allclose(red[k], KT[k], rtol=1e-12, atol=0), k
    # rwgt sums to 1 over each reduced interval (weights renormalised per interval)
    rw = rwgt_table(REF)
    ngm = REF["ngm"]
    for b in range(16):
        for igc in range(1, NG[b] + 1):
            sel = (ngm[b * 16:(b + 1) * 16] == igc)
            assert abs(rw[b * 16:(b + 1) * 16][sel].sum() - 1.0) < 1e-12 or NG[b] == 16


def test_monotone_in_g_before_perturbation():
    """The synthetic major-absorber tables grow with g (weak to strong lines)."""
    for b in range(1, 17):
        ka = KT[f"b{b:02d}.ka"]
        med = np.median(ka.reshape(-1, ka.shape[-1]), axis=0)
        assert np.all(np.diff(med) > 0), b
