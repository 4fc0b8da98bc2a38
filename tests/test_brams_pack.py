"""The CPU restatement of BRAMS's column packing and tendency write-back
(oracle/brams_pack.py, rtm_driver.f90:978-1231 and :1443-1456): column order,
a packed state the FP64 solver accepts, and the write-back's level copies."""
import os
import sys

import numpy as np

from brams_fields import brams_fields, ozone

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import brams_pack as BP  # noqa: E402


def test_columns_run_j_outer_i_inner():
    i, j = BP.column_index(7, 5, 2, 4, 3, 5)
    assert list(zip(i[:4], j[:4])) == [(1, 2), (2, 2), (3, 2), (1, 3)]
    assert i.size == 9


def test_packed_state_feeds_the_solver():
    import pyoracle

    f = brams_fields(30, 6, 5, seed=11)
    st = BP.pack_lw(f, 2, 5, 1, 4)
    ncol, nlay = st["play"].shape
    assert (ncol, nlay) == (16, 29)
    assert (np.diff(st["plev"], axis=1) < 0).all() and (np.diff(st["play"], axis=1) < 0).all()
    assert (st["plev"][:, :-1] > st["play"]).all() and (st["play"] > st["plev"][:, 1:]).all()
    assert (st["tlay"] > 180.0).all() and (st["tlay"] < 320.0).all()
    assert np.allclose(st["emis"], 1.0 - f["albedt"][1:5, 0:4].T.ravel()[:, None], atol=1e-6)
    assert (st["rei"] >= 5.0).all() and (st["rei"] <= 140.0).all()
    st["o3vmr"] = ozone(st["play"])
    st["tauaer"] = np.zeros((ncol, nlay, 16), order="F")
    st = {k: np.asfortranarray(v) for k, v in st.items()}
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=5)
    out = pyoracle.rrtmg_lw(st, mc, icld=3)
    assert np.isfinite(out["hr"]).all() and (out["dflx"][:, 0] > 100.0).all()
    fthrd, rlong = BP.unpack_lw(out["hr"], out["dflx"], None, 30, 6, 5, 2, 5, 1, 4)
    assert np.isfinite(fthrd).all()
    assert np.array_equal(rlong[1:5, 0:4].T.ravel(), out["dflx"][:, 0].astype(np.float32))


def test_write_back_copies_the_end_levels_and_leaves_other_columns():
    mzp, mxp, myp = 8, 4, 3
    rs = np.random.default_rng(3)
    hr = rs.normal(0.0, 2.0, (6, mzp - 1))
    sw = rs.normal(0.0, 1.0, (6, mzp - 1))
    dflx = rs.uniform(200.0, 400.0, (6, mzp))
    f0 = np.full((mzp, mxp, myp), 7.0, np.float32)
    r0 = np.full((mxp, myp), 9.0, np.float32)
    fthrd, rlong = BP.unpack_lw(hr, dflx, sw, mzp, mxp, myp, 2, 4, 2, 3, f0, r0)
    col = fthrd[:, 1, 1]  # first packed column (i = 2, j = 2)
    assert np.array_equal(col[1:mzp - 1], ((sw[0, :mzp - 2] + hr[0, :mzp - 2]) / 86400.0).astype(np.float32))
    assert col[0] == col[1] and col[mzp - 1] == col[mzp - 2]
    assert (fthrd[:, 0, :] == 7.0).all() and (fthrd[:, :, 0] == 7.0).all()
    assert rlong[0, 0] == 9.0 and rlong[1, 1] == np.float32(dflx[0, 0])


def test_shortwave_inputs_and_surface_flux():
    """coszen and the four albedos per packed column (albedos 0 on the first
    call), and rshort from the surface downward shortwave flux, 0 below
    0.5 W m-2, other columns untouched."""
    rs = np.random.default_rng(4)
    cosz = rs.uniform(-0.3, 1.0, (5, 4)).astype(np.float32)
    albedt = rs.uniform(0.05, 0.6, (5, 4)).astype(np.float32)
    p = BP.pack_sw(cosz, albedt, 2, 4, 2, 3)
    assert p["coszen"][0] == np.float64(cosz[1, 1]) and p["coszen"].size == 6
    for k in ("asdir", "asdif", "aldir", "aldif"):
        assert np.array_equal(p[k], p["asdir"]) and p[k][3] == np.float64(albedt[1, 2])
    p0 = BP.pack_sw(cosz, albedt, 2, 4, 2, 3, firsttime=True)
    assert (p0["asdir"] == 0.0).all() and np.array_equal(p0["coszen"], p["coszen"])
    swdflx = np.array([[800.0], [0.49], [0.5], [1e-9], [350.25], [12.0]])
    r = BP.unpack_sw(swdflx, 5, 4, 2, 4, 2, 3, np.full((5, 4), 3.0, np.float32))
    assert r[1, 1] == np.float32(800.0) and r[2, 1] == 0.0 and r[3, 1] == np.float32(0.5) and r[1, 2] == 0.0
    assert r[0, 0] == 3.0 and r[4, 3] == 3.0
