"""The oracle's non-McICA random-overlap path (rrtmg_lw_rad.nomcica.f90 with
icld 1: cldprop on band-level clouds, then rtrn): overcast-or-clear layers
give the McICA path's fluxes with every sub-column equal to the layer's
cloud, clear-sky fluxes do not see the clouds, and with one cloudy layer over
a black surface the fluxes are affine in its cloud fraction, as rtrn's
per-layer update is."""
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


def test_other_overlap_methods_are_refused():
    L = pyoracle.lib()
    null = [None] * 24
    rc = L.ora_rrtmg_lw_rtrn(C.c_int(1), C.c_int(10), C.c_int(2), C.c_int(1), *null[:16],
                             C.c_int(2), C.c_int(3), C.c_int(1), *null[:15])
    assert rc == 7  # ERR_ICLD: rtrnmr is not restated
