"""GPU parity: the CUDA library through its C ABI against the FP64 oracle.

Tolerances are the ones the solver is specified to: upward/downward fluxes
within 0.05 W m-2 and heating rates within 0.01 K/day of the FP64 oracle,
McICA sub-column draws bit-identical.
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu

FLUX_TOL = 0.05  # W m-2
HR_TOL = 0.01  # K/day


def _case(ncol, nlay, seed, **kw):
    spec = ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, **kw)
    st = make_state(spec)
    tauc = pyoracle.cldprop_columns(st)
    return st, tauc


def _compare(out, ref, idrv=1):
    errs = {}
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        errs[k] = float(np.abs(out[k] - ref[k]).max())
    for k in ("hr", "hrc"):
        errs[k] = float(np.abs(out[k] - ref[k]).max())
    if idrv == 1:
        for k in ("duflx_dt", "duflxc_dt"):
            errs[k] = float(np.abs(out[k] - ref[k]).max())
    return errs


def _assert_tol(errs):
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert errs[k] <= FLUX_TOL, (k, errs)
    for k in ("hr", "hrc"):
        assert errs[k] <= HR_TOL, (k, errs)
    for k in ("duflx_dt", "duflxc_dt"):
        if k in errs:
            assert errs[k] <= 1e-3, (k, errs)  # W m-2 K-1


@pytest.mark.parametrize("icld", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("irng", [0, 1])
def test_mcica_percolumn_bitexact(ctx, icld, irng):
    st, tauc = _case(24, 30, seed=11)
    gpu = ctx.mcica_subcol_lw(st, tauc, icld=icld, permuteseed=7, irng=irng, alpha=_alpha(st) if icld >= 4 else None,
                              seed_per_column=True)
    ref = {k: np.zeros_like(gpu[k]) for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl")}
    for i in range(st["play"].shape[0]):
        sub = {k: np.asfortranarray(st[k][i:i + 1]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")}
        al = np.asfortranarray(_alpha(st)[i:i + 1]) if icld >= 4 else None
        r = pyoracle.mcica_subcol_lw(sub, np.asfortranarray(tauc[:, i:i + 1]), icld, 7 + i, irng, al)
        for k in ref:
            ref[k][:, i] = r[k][:, 0]
    for k in ref:
        assert np.array_equal(gpu[k], ref[k]), k


@pytest.mark.parametrize("icld", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("irng", [0, 1])
def test_mcica_single_call_bitexact(ctx, icld, irng):
    st, tauc = _case(16, 20, seed=12)
    al = _alpha(st) if icld >= 4 else None
    gpu = ctx.mcica_subcol_lw(st, tauc, icld=icld, permuteseed=3, irng=irng, alpha=al, seed_per_column=False)
    ref = pyoracle.mcica_subcol_lw(st, tauc, icld, 3, irng, al)
    for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "reicmcl", "relqmcl"):
        assert np.array_equal(gpu[k], ref[k]), k


def _alpha(st):
    ncol, nlay = st["play"].shape
    a = np.exp(-np.linspace(0.1, 2.0, nlay))[None, :] * np.ones((ncol, 1))
    a[:, 0] = 0.0
    return np.asfortranarray(a)


@pytest.mark.parametrize("nlay,ptop", [(38, 10.0), (45, 10.0), (60, 5.0)])
def test_rrtmg_lw_parity(ctx, nlay, ptop):
    st, tauc = _case(64, nlay, seed=100 + nlay, ptop=ptop, t_noise=4.0, h2o_sigma=0.5)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    ref = pyoracle.rrtmg_lw(st, mc, nthreads=4)
    out = ctx.rrtmg_lw(st, mc)
    _assert_tol(_compare(out, ref))


def test_fractional_subcolumn_cells(ctx):
    """Caller sub-columns are not only 0 or 1: rtrnmc gives a cell whose
    cldfmcl is a fraction no cloud optical depth but weights its cloudy
    source by the fraction (rrtmg_lw_rtrnmc.f90:300-312, 380-455); cells at
    and below cldmin and fractions next to cloudy cells of the same layer go
    through the transfer's cloud hand-over as the fraction itself."""
    st, tauc = _case(48, 45, seed=321, t_noise=3.0, h2o_sigma=0.4, cloud_prob=0.8)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=3)
    rng = np.random.default_rng(9)
    cf = np.array(mc["cldfmcl"], order="F")
    pick = rng.uniform(size=cf.shape) < 0.15
    vals = rng.choice(np.array([0.3, 0.75, 1e-20, 1e-25, 0.999]), size=cf.shape)
    cf[pick] = vals[pick]
    mc = dict(mc)
    mc["cldfmcl"] = np.asfortranarray(cf)
    assert ((cf > 0) & (cf < 1)).sum() > 1000 and (cf == 1.0).sum() > 1000
    ref = pyoracle.rrtmg_lw(st, mc, nthreads=4)
    out = ctx.rrtmg_lw(st, mc)
    _assert_tol(_compare(out, ref))


def test_clear_sky_equals_total_without_clouds(ctx):
    st, tauc = _case(32, 45, seed=5)
    st["cldfrac"][:] = 0.0
    mc = pyoracle.mcica_per_column(st, tauc * 0, icld=3, base_seed=1)
    out = ctx.rrtmg_lw(st, mc)
    for a, b in (("uflx", "uflxc"), ("dflx", "dflxc"), ("hr", "hrc"), ("duflx_dt", "duflxc_dt")):
        assert np.array_equal(out[a], out[b]), (a, b)
    ref = pyoracle.rrtmg_lw(st, mc)
    _assert_tol(_compare(out, ref))


def test_icld0_and_idrv0(ctx):
    st, tauc = _case(16, 38, seed=9)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    ref = pyoracle.rrtmg_lw(st, mc, icld=0, idrv=0)
    out = ctx.rrtmg_lw(st, None, icld=0, idrv=0)
    errs = _compare(out, ref, idrv=0)
    _assert_tol(errs)
    assert np.all(out["duflx_dt"] == 0.0)  # not written when idrv == 0


def test_icld_clamped_like_reference(ctx):
    st, tauc = _case(8, 38, seed=3)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    out = ctx.rrtmg_lw(st, mc, icld=7)
    assert out["icld"] == 2


def test_leading_dimension_and_column_independence(ctx):
    """Wider caller allocations (ld > ncol) give the same columns as tight ones."""
    import ctypes as C

    st, tauc = _case(20, 38, seed=21)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    tight = ctx.rrtmg_lw(st, mc)
    ncol, nlay = st["play"].shape
    ld = ncol + 5
    pad = {}
    for k in ("play", "plev", "tlay", "tlev", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
              "cfc11vmr", "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis"):
        a = np.full((ld, st[k].shape[1]), 7.0, order="F")
        a[:ncol] = st[k]
        pad[k] = a
    pad["tsfc"] = np.concatenate([st["tsfc"], np.full(5, 7.0)])
    ta = np.zeros((ld, nlay, 16), order="F")
    pad["tauaer"] = ta
    for k in ("cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl"):
        a = np.zeros((140, ld, nlay), order="F")
        a[:, :ncol] = mc[k]
        pad[k] = a
    for k in ("reicmcl", "relqmcl"):
        a = np.full((ld, nlay), 10.0, order="F")
        a[:ncol] = mc[k]
        pad[k] = a
    ldo = ncol + 3
    outs = {k: np.full((ldo, nlay + 2), -1.0, order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    outs["hr"] = np.full((ldo, nlay + 1), -1.0, order="F")
    outs["hrc"] = np.full((ldo, nlay + 1), -1.0, order="F")
    rc = ctx.rrtmg_lw_host_ptrs(ncol, nlay, {**pad, **outs}, ld_in=ld, ld_out=ldo)
    assert rc == 0
    for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
        assert np.array_equal(outs[k][:ncol, :nlay + 1], tight[k]), k
        assert np.all(outs[k][ncol:] == -1.0) and np.all(outs[k][:, nlay + 1] == -1.0)
    for k in ("hr", "hrc"):
        assert np.array_equal(outs[k][:ncol, :nlay], tight[k]), k


def test_stop_conditions_reported(ctx):
    from brams_gb300.rrtmg_lw import RrtmgLwError

    st, tauc = _case(8, 38, seed=4)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    bad = dict(mc)
    bad["relqmcl"] = np.asfortranarray(np.full_like(mc["relqmcl"], 70.0))  # > 60 um
    if np.any((mc["cldfmcl"] > 0) & (mc["clwpmcl"] > 0)):
        with pytest.raises(RrtmgLwError) as e:
            ctx.rrtmg_lw(st, bad)
        assert e.value.code == 6
    with pytest.raises(RrtmgLwError) as e:
        ctx.rrtmg_lw(st, mc, inflglw=1)
    assert e.value.code in (2, -1)
    rev = {k: (np.asfortranarray(v[:, ::-1]) if k in ("play", "tlay") else v) for k, v in st.items()}
    with pytest.raises(RrtmgLwError) as e:
        ctx.rrtmg_lw(rev, mc)
    assert e.value.code == 9
