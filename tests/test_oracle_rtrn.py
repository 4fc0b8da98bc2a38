"""The oracle's non-McICA paths (rrtmg_lw_rad.nomcica.f90: cldprop on
band-level clouds, then rtrn for icld 1 and rtrnmr otherwise).

Random overlap (rtrn): overcast-or-clear layers give the McICA path's fluxes
with every sub-column equal to the layer's cloud, clear-sky fluxes do not see
the clouds, and with one cloudy layer over a black surface the fluxes are
affine in its cloud fraction, as rtrn's per-layer update is.

Maximum/random overlap (rtrnmr): where overlap cannot matter (overcast or
clear layers, a single cloudy layer) it agrees with rtrn to the precision of
the transmittance tables (rtrnmr takes the total layer transmittance from the
table, rtrn multiplies the gas table value by the exact cloud one); where it
matters (vertically extended partial clouds) the cover seen from the surface
is smaller than random overlap's; icld 0 is clear sky, icld 3 is icld 2, and
other values become 2, as in the driver (:456)."""
import ctypes as C

import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state

OUTS = ("uflx", "dflx", "uflxc", "dflxc", "hr", "hrc", "duflx_dt", "duflxc_dt")


def _state(seed, ncol=12, nlay=38):
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=2.0, h2o_sigma=0.3))
    return {k: np.asfortranarray(v) for k, v in st.items()}


def _mcica_equal_to_layers(st):
    cf = st["cldfrac"]
    ncol, nlay = cf.shape
    rep = lambda a: np.asfortranarray(np.broadcast_to(a[None], (140, ncol, nlay)).copy())
    return {"cldfmcl": rep(cf), "ciwpmcl": rep(st["ciwp"] * cf), "clwpmcl": rep(st["clwp"] * cf),
            "taucmcl": np.zeros((140, ncol, nlay), order="F"),
            "reicmcl": np.asfortranarray(st["rei"]), "relqmcl": np.asfortranarray(st["rel"])}


def test_overcast_or_clear_layers_match_mcica():
    st = _state(31)
    st["cldfrac"] = np.asfortranarray((st["cldfrac"] > 0).astype(np.float64))
    assert st["cldfrac"].sum() > 10
    a = pyoracle.rrtmg_lw_rtrn(st)
    b = pyoracle.rrtmg_lw(st, _mcica_equal_to_layers(st), icld=3)
    for k in OUTS:
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-12), (k, float(np.abs(a[k] - b[k]).max()))
    assert not np.allclose(a["dflx"], a["dflxc"])  # the clouds are seen


def test_clear_sky_fluxes_do_not_see_the_clouds():
    st = _state(32)
    a = pyoracle.rrtmg_lw_rtrn(st)
    clear = dict(st)
    clear["cldfrac"] = np.zeros_like(st["cldfrac"], order="F")
    b = pyoracle.rrtmg_lw_rtrn(clear)
    for k in ("uflxc", "dflxc", "hrc", "duflxc_dt"):
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-12), k
    for k in ("uflx", "dflx", "hr"):
        assert np.allclose(b[k], b[k.replace("flx", "flxc") if "flx" in k else "hrc"], rtol=1e-12, atol=1e-12), k


def test_fluxes_are_affine_in_one_layers_cloud_fraction():
    st = _state(33, ncol=6)
    lay = 8
    base = dict(st)
    base["cldfrac"] = np.zeros_like(st["cldfrac"], order="F")
    base["clwp"] = np.zeros_like(st["clwp"], order="F")
    base["ciwp"] = np.zeros_like(st["ciwp"], order="F")
    base["clwp"][:, lay] = 40.0
    base["emis"] = np.ones_like(st["emis"], order="F")  # no surface reflection: the downward
    # radiance through the cloud would come back up through it (quadratic in f)
    outs = {}
    for f in (0.2, 0.5, 0.8):
        s = dict(base)
        s["cldfrac"] = base["cldfrac"].copy(order="F")
        s["cldfrac"][:, lay] = f
        outs[f] = pyoracle.rrtmg_lw_rtrn(s)
    for k in ("uflx", "dflx", "hr", "duflx_dt"):
        mid = 0.5 * (outs[0.2][k] + outs[0.8][k])
        scale = np.abs(outs[0.5][k]).max()
        assert np.abs(outs[0.5][k] - mid).max() <= 1e-10 * scale, k
        assert np.abs(outs[0.8][k] - outs[0.2][k]).max() > 1e-4 * scale, k  # the fraction matters


def _cloudy_state(seed, ncol=12, nlay=38):
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=2.0, h2o_sigma=0.3, cloud_prob=0.6))
    return {k: np.asfortranarray(v) for k, v in st.items()}


TABLE_TOL = 0.02  # W m-2: the two ways of forming a cloudy layer's transmittance


def test_maxrandom_equals_random_for_overcast_or_clear_layers():
    st = _cloudy_state(41)
    st["cldfrac"] = np.asfortranarray((st["cldfrac"] > 0).astype(np.float64))
    a = pyoracle.rrtmg_lw_nomcica(st, 1)
    b = pyoracle.rrtmg_lw_nomcica(st, 2)
    assert b["icld"] == 2
    for k in ("uflx", "dflx"):
        assert np.abs(a[k] - b[k]).max() <= TABLE_TOL, k
    for k in ("uflxc", "dflxc", "duflxc_dt"):
        assert np.array_equal(a[k], b[k]), k


def test_maxrandom_equals_random_for_one_cloudy_layer():
    st = _cloudy_state(42, ncol=6)
    lay = 10
    st["cldfrac"] = np.zeros_like(st["cldfrac"], order="F")
    st["cldfrac"][:, lay] = np.linspace(0.1, 0.9, 6)
    st["clwp"] = np.zeros_like(st["clwp"], order="F")
    st["clwp"][:, lay] = 60.0
    a = pyoracle.rrtmg_lw_nomcica(st, 1)
    b = pyoracle.rrtmg_lw_nomcica(st, 2)
    for k in ("uflx", "dflx"):
        assert np.abs(a[k] - b[k]).max() <= TABLE_TOL, k
    assert np.abs(a["dflx"] - a["dflxc"]).max() > 5.0  # the cloud matters


def test_maxrandom_overlap_shows_less_cloud_than_random():
    """Two adjacent thick layers with equal partial cover: maximum overlap
    gives cover f, random 1-(1-f)^2, so the clouds' surface-forcing is
    smaller under rtrnmr, and roughly in that ratio."""
    st = _cloudy_state(43, ncol=6)
    st["cldfrac"] = np.zeros_like(st["cldfrac"], order="F")
    st["clwp"] = np.zeros_like(st["clwp"], order="F")
    st["ciwp"] = np.zeros_like(st["ciwp"], order="F")
    f = 0.5
    for lay in (4, 5):
        st["cldfrac"][:, lay] = f
        st["clwp"][:, lay] = 200.0
    a = pyoracle.rrtmg_lw_nomcica(st, 1)
    b = pyoracle.rrtmg_lw_nomcica(st, 2)
    fa = a["dflx"][:, 0] - a["dflxc"][:, 0]
    fb = b["dflx"][:, 0] - b["dflxc"][:, 0]
    assert (fa > 1.0).all() and (fb > 1.0).all()
    ratio = fb / fa
    assert (np.abs(ratio - f / (1 - (1 - f) ** 2)) < 0.1).all(), ratio


def test_clear_and_overlap_flag_handling():
    st = _cloudy_state(44)
    z = pyoracle.rrtmg_lw_nomcica(st, 0)
    for k in ("uflx", "dflx", "hr"):
        kc = "hrc" if k == "hr" else k + "c"
        assert np.array_equal(z[k], z[kc]), k
    r = pyoracle.rrtmg_lw_nomcica(st, 1)
    for k in ("uflxc", "dflxc", "hrc"):
        assert np.array_equal(z[k], r[k]), k
    two, three, seven, neg = (pyoracle.rrtmg_lw_nomcica(st, i) for i in (2, 3, 7, -1))
    assert seven["icld"] == 2 and neg["icld"] == 2 and three["icld"] == 3
    for k in OUTS:
        assert np.array_equal(two[k], three[k]) and np.array_equal(two[k], seven[k]), k
    assert np.abs(two["dflx"] - r["dflx"]).max() > 1.0  # the overlap assumption matters here


def test_maxrandom_fluxes_are_continuous_in_cloud_fraction():
    """rtrnmr switches overlap branches where neighbouring fractions cross;
    the fluxes stay continuous through those switches."""
    st = _cloudy_state(45, ncol=1)
    st["cldfrac"] = np.zeros_like(st["cldfrac"], order="F")
    st["clwp"] = np.zeros_like(st["clwp"], order="F")
    st["ciwp"] = np.zeros_like(st["ciwp"], order="F")
    prof = [0.3, 0.6, 0.45, 0.7]
    for i, lay in enumerate(range(6, 10)):
        st["cldfrac"][0, lay] = prof[i]
        st["clwp"][0, lay] = 80.0
    outs = []
    xs = np.linspace(0.2, 0.8, 121)  # layer 8's fraction sweeps past 0.3, 0.6 and 0.7
    for x in xs:
        s = dict(st)
        s["cldfrac"] = st["cldfrac"].copy(order="F")
        s["cldfrac"][0, 8] = x
        outs.append(pyoracle.rrtmg_lw_nomcica(s, 2)["dflx"][0])
    d = np.abs(np.diff(np.array(outs), axis=0)).max(axis=1)
    assert d.max() < 10 * np.median(d) + 1e-3, d.max()
