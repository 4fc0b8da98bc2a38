"""Inputs placed exactly on setcoef's and taumol's decision boundaries.

The reference takes these decisions in double precision:

* jp = int(36 - 5*(log(p) + 0.04)), jt/jt1 = int(3 + (T - tref)/15)
  (rrtmg_lw_setcoef.f90:276-306);
* laytrop: log(p) > 4.56 (:312);
* specparm < 0.125 and > 0.875, the switch to the three-point stencil in the
  binary-species eta (rrtmg_lw_taumol.f90:582-611), and js = 1 + int(8 *
  specparm) (:517-522).

The GPU computes them in fp32 and re-takes them in fp64 near a boundary.  The
columns here put layers on those boundaries (and one part in 1e7 either side)
and compare taumol band by band and the fluxes with the FP64 oracle; the
tests also assert that the data reaches both sides of each switch.
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state
from brams_gb300.tables_io import read_tables

NGS0 = [0, 10, 22, 38, 52, 68, 76, 88, 96, 108, 114, 122, 130, 134, 136, 138, 140]
FLUX_TOL, HR_TOL = 0.05, 0.01


def _tables():
    import os

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return read_tables(os.path.join(root, "brams_gb300", "data", "lw_ref_tables.gblw"))


def _jp(p):
    return np.clip((36.0 - 5 * (np.log(p) + 0.04)).astype(np.int64), 1, 58)


def _boundary_state():
    """16 columns x 38 layers with layers on the decision boundaries."""
    t = _tables()
    chi, tref = np.asarray(t["chi_mls"]), np.asarray(t["tref"])
    st = make_state(ProfileSpec(ncol=16, nlay=38, seed=211, t_noise=2.0, h2o_sigma=0.3))
    ncol, nlay = st["play"].shape
    # columns 0-2: every fourth layer's pressure on a jp boundary (exactly, and
    # one part in 1e7 above and below)
    for c, eps in ((0, 0.0), (1, 1e-7), (2, -1e-7)):
        for lay in range(1, nlay - 1, 4):
            x = 36.0 - 5 * (np.log(st["play"][c, lay]) + 0.04)
            k = np.round(x)
            st["play"][c, lay] = np.exp((36.0 - k) / 5 - 0.04) * (1.0 + eps)
    # columns 3-5: one layer on the laytrop switch log(p) = 4.56
    for c, eps in ((3, 0.0), (4, 1e-9), (5, -1e-9)):
        lay = int(np.argmin(np.abs(np.log(st["play"][c]) - 4.56)))
        st["play"][c, lay] = np.exp(4.56 + eps)
    # columns 6-8: layer temperatures on jt boundaries (T = tref(jp) + 15 m)
    for c, eps in ((6, 0.0), (7, 1e-6), (8, -1e-6)):
        jp = _jp(st["play"][c])
        for lay in range(nlay):
            m = np.round((st["tlay"][c, lay] - tref[jp[lay] - 1]) / 15.0)
            st["tlay"][c, lay] = tref[jp[lay] - 1] + 15.0 * m + eps
    # columns 9-15: water vapour putting band 3's H2O/CO2 specparm on 0.125,
    # 0.875 and 3/8 (a js boundary) in the lower atmosphere
    for c, (target, eps) in zip(range(9, 16), ((0.125, 0.0), (0.125, 1e-7), (0.125, -1e-7), (0.875, 0.0),
                                               (0.875, 1e-7), (0.875, -1e-7), (0.375, 0.0))):
        jp = _jp(st["play"][c])
        for lay in range(nlay):
            if np.log(st["play"][c, lay]) <= 4.56:
                continue
            r = chi[0, jp[lay] - 1] / chi[1, jp[lay] - 1]
            p = target * (1.0 + eps)
            st["h2ovmr"][c, lay] = r * st["co2vmr"][c, lay] * p / (1.0 - p)
    st["tauaer"] = np.asfortranarray(np.random.default_rng(5).uniform(0.0, 0.02, (ncol, nlay, 16)))
    return st


def _specparm_band3(st, c):
    """band 3's lower-atmosphere specparm per layer, as the oracle computes it."""
    t = _tables()
    chi = np.asarray(t["chi_mls"])
    jp = _jp(st["play"][c])
    h, co2 = st["h2ovmr"][c], st["co2vmr"][c]
    r = chi[0, jp - 1] / chi[1, jp - 1]
    lower = np.log(st["play"][c]) > 4.56
    return (h / (h + r * co2))[lower]


def test_boundaries_are_reached():
    st = _boundary_state()
    sp = np.concatenate([_specparm_band3(st, c) for c in range(9, 16)])
    assert (sp < 0.125).any() and (sp > 0.875).any() and ((sp >= 0.125) & (sp <= 0.875)).any()
    plog = np.log(st["play"])
    for c in (3, 4, 5):  # a layer on each side of the switch, and one on it
        assert (plog[c] > 4.56).any() and (plog[c] <= 4.56).any()
    assert np.abs(plog[4] - 4.56).min() < 1e-8 and np.abs(plog[5] - 4.56).min() < 1e-8


@pytest.mark.gpu
def test_taumol_on_boundaries(ctx):
    st = _boundary_state()
    ncol, nlay = st["play"].shape
    taut, fracs = ctx.gas_optics_diag(st)
    mc0 = {k: np.zeros((140, ncol, nlay), order="F") for k in ("cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl")}
    mc0["reicmcl"] = np.asfortranarray(st["rei"])
    mc0["relqmcl"] = np.asfortranarray(st["rel"])
    worst = {}
    for icol in range(ncol):
        im = pyoracle.column_intermediates(st, mc0, icol + 1, icld=0)
        rt, rf = im["taut"], im["fracs"]
        gt, gf = taut[icol].astype(np.float64), fracs[icol].astype(np.float64)
        for b in range(16):
            g0, g1 = NGS0[b], NGS0[b + 1]
            et = np.abs(gt[:, g0:g1] - rt[:, g0:g1]) / (np.abs(rt[:, g0:g1]) + 1e-6)
            ef = np.abs(gf[:, g0:g1] - rf[:, g0:g1])
            worst[(icol, b + 1)] = max(float(et.max()), float(ef.max()))
    bad = {k: v for k, v in worst.items() if v > 2e-4}
    assert not bad, f"(column, band) with relative taut/frac error > 2e-4: {bad}"


@pytest.mark.gpu
def test_fluxes_on_boundaries(ctx):
    st = _boundary_state()
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=17)
    ref = pyoracle.rrtmg_lw(st, mc, nthreads=4)
    out = ctx.rrtmg_lw(st, mc)
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= FLUX_TOL, k
    for k in ("hr", "hrc"):
        assert np.abs(out[k] - ref[k]).max() <= HR_TOL, k
