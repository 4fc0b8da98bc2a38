"""BRAMS's ozone climatology for the packed columns: the library's host
function (gb_rtm_ozone_lw) against the scalar restatement in
oracle/brams_ozone.py, the extracted table against values of the driver's
source, and the restatement against the climatology's own limits."""
import os
import sys

import numpy as np

from brams_gb300 import rrtmg_lw as R
from brams_gb300.tables_io import read_tables

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import brams_ozone as BO  # noqa: E402

TAB = read_tables(os.path.join(R.DATA_DIR, "brams_ozone.gblw"))


def _plev(ncol, mzp, seed):
    rs = np.random.default_rng(seed)
    ps = rs.uniform(950.0, 1020.0, ncol)
    z = np.cumsum(rs.uniform(150.0, 600.0, (ncol, mzp)), axis=1) - 150.0
    z[:, 0] = 0.0
    return ps[:, None] * np.exp(-z / 7500.0)


def test_table_holds_the_drivers_values():
    oz, sig = TAB["ozone"], TAB["ozsig"]
    assert oz.shape == (18, 37, 4) and sig.shape == (18,)
    # rtm_driver.f90: the first value of ozone(1:18, 1:6, 1), the last of
    # ozone(1:18, 37, 4), and the ends of ozsig
    assert oz[0, 0, 0] == 0.068467 and oz[17, 36, 3] == 0.000515 and oz[0, 36, 3] == 0.074229
    assert sig[0] == 0.020747 and sig[17] == 0.995004
    assert (np.diff(sig) > 0).all() and (oz > 0).all()


def test_library_matches_the_restatement():
    oz = R.Ozone()
    for mzp, doy, seed in ((40, 1, 1), (33, 172, 2), (61, 365, 3), (18, 700, 4)):
        plev = _plev(23, mzp, seed)
        glat = np.random.default_rng(seed).uniform(-89.9, 89.9, 23).astype(np.float32)
        got = oz.o3vmr(plev, glat, doy)
        want = np.array(BO.o3vmr_columns(TAB["ozone"], TAB["ozsig"], plev, glat, doy))
        assert np.array_equal(got, want), (mzp, doy, float(np.abs(got - want).max()))
        assert (got > 0).all()
    oz.close()


def test_restatement_returns_the_table_on_its_nodes():
    oz, sig = TAB["ozone"], TAB["ozsig"]
    # date = rlag: rang = 0, so the seasonal harmonic gives season 1; latitude
    # 40 N: flat = 8, la = ll = 11, rate = 0
    colrad = BO.PAI * (1.0 - (40.0 + 90.0) / 180.0)
    sigmid = [0.0] + list(sig[::-1])  # layers at the table's own sigma levels, surface first
    o3l = BO.getoz(oz, sig, 18, sigmid, colrad, BO.RLAG, True)
    want = 1.0e-4 * oz[:, 10, 0]
    assert np.allclose(o3l, want, rtol=1e-9, atol=0.0)


def test_restatement_against_hand_computed_values():
    """getoz_rrtm (rtm_driver.f90:2638-2823) without interpolation at
    latitudes between the table's 5-degree bands and at dates past one year
    (doy > 365 wraps), against values computed once with the driver's
    formulas written out by hand (seasonal harmonics of the four seasons at
    the two bracketing latitude rows, blended by `rate`)."""
    oz, sig = TAB["ozone"], TAB["ozsig"]
    cases = {  # (glat, doy): {level k: 1e-4 * ozone at the column's latitude and date}
        (37.3, 400): {1: 1.0190352056605059e-05, 9: 5.5347364120273215e-08, 18: 3.184062131023349e-08},
        (-12.7, 59): {1: 1.0311197986310936e-05, 9: 4.600614880396558e-08, 18: 6.626378266628427e-09},
        (81.1, 730): {1: 6.846653122921635e-06, 9: 9.63757620967659e-08, 18: 2.819129576826978e-08},
    }
    for (glat, doy), want in cases.items():
        colrad = BO.PAI * (1.0 - (glat + 90.0) / 180.0)
        o3l = BO.getoz(oz, sig, 18, [0.0] * 19, colrad, float(doy), False)
        for k, v in want.items():
            assert abs(o3l[k - 1] - v) <= 1e-12 * abs(v), (glat, doy, k)


def test_eighteen_levels_still_interpolate():
    """The driver skips the interpolation only when the column's sigma levels
    equal the table's within 1e-4 (rtm_driver.f90:1130-1140); sig(1) is 1 by
    construction and ozsig(18) = 0.995004, so a column of 18 levels is always
    interpolated: its ozone equals the restatement's interpolated values."""
    plev = _plev(5, 18, 11)
    glat = np.array([37.3, -12.7, 81.1, 0.0, -60.0], dtype=np.float32)
    oz = R.Ozone()
    got = oz.o3vmr(plev, glat, 400)
    oz.close()
    want = np.array(BO.o3vmr_columns(TAB["ozone"], TAB["ozsig"], plev, glat, 400))
    assert np.array_equal(got, want)
