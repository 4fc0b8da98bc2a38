"""RRTMG_SW: the tables, the FP64 oracle and the GPU path.

Tables: ``brams_gb300/data/sw_tables.gbsw`` holds the reference's own
k-distribution data (rrtmg_sw_k_g.f90) reduced to 112 g-points with the
reference's reduction (rrtmg_sw_init.f90:492-1689); the reduction keeps the
solar source of every band (plain sums) and every weighted table is a convex
combination of the original g-points (the weights of each reduced g-point
sum to 1).

Oracle pins (project-made; the reference has no tests or fixtures):
* the incoming flux at the top is coszen x the Kurucz source (1368.22 W m-2)
  x the Earth-Sun factor, for every column;
* over a grey surface the clear-sky up/down flux ratio at the surface is the
  albedo;
* a purely scattering atmosphere (no absorbers, Rayleigh only) conserves
  energy: the net flux is the same at every level and the heating rates
  vanish;
* clouds only add reflection: total-sky TOA upward flux >= clear-sky.

GPU, both precisions of the column kernel: with everything in FP64 the
library matches the oracle at rounding level (fluxes within 1e-6 W m-2,
heating rates within 1e-8 K/day); with the gas optics, cloud optics and
two-stream solution in FP32 (FP64 flux sums and heating rates) within
0.05 W m-2 and 0.01 K/day.  Cases: clear and McICA-cloudy columns, every ice
option, the direct cloud-optics input (inflag 0), aerosols, day-of-year and
solar-constant scaling, low sun and night columns, wide leading dimensions,
and the radius bounds the reference stops on, decided on the double inputs
in both precisions.
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state
from brams_gb300.tables_io import read_tables

NGS = [6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12]


def _tables():
    import os

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return read_tables(os.path.join(root, "brams_gb300", "data", "sw_tables.gbsw"))


def sw_state(ncol=8, nlay=45, seed=5, cloud_prob=0.5):
    """A generator profile with the SW inputs: albedos, solar zenith, aerosols."""
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=3.0, h2o_sigma=0.4, cloud_prob=cloud_prob))
    rng = np.random.default_rng(seed)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        st[k] = rng.uniform(0.05, 0.6, ncol)
    st["coszen"] = rng.uniform(0.05, 1.0, ncol)
    st["tauaer_sw"] = np.asfortranarray(rng.uniform(0.0, 0.05, (ncol, nlay, 14)))
    st["ssaaer_sw"] = np.asfortranarray(rng.uniform(0.8, 0.99, (ncol, nlay, 14)))
    st["asmaer_sw"] = np.asfortranarray(rng.uniform(0.5, 0.8, (ncol, nlay, 14)))
    return st


def sw_mcica(st, seed=1, iceflag=3, inflag=2):
    """McICA arrays (112, ncol, nlay): each g-point's cell cloudy with the
    layer's fraction; water paths and radii of the layer; for inflag 0, cloud
    optical depth, single-scattering albedo, asymmetry and forward fraction."""
    ncol, nlay = st["play"].shape
    rng = np.random.default_rng(seed)
    cf = (rng.uniform(size=(112, ncol, nlay)) < st["cldfrac"][None]).astype(np.float64)
    mc = {"cldfmcl": np.asfortranarray(cf),
          "ciwpmcl": np.asfortranarray(cf * st["ciwp"][None]),
          "clwpmcl": np.asfortranarray(cf * st["clwp"][None]),
          "taucmcl": np.asfortranarray(cf * rng.uniform(0.5, 20.0, cf.shape)),
          "ssacmcl": np.asfortranarray(rng.uniform(0.9, 0.9999, cf.shape)),
          "asmcmcl": np.asfortranarray(rng.uniform(0.7, 0.9, cf.shape)),
          "fsfcmcl": np.asfortranarray(rng.uniform(0.0, 0.5, cf.shape)),
          "relqmcl": np.asfortranarray(rng.uniform(4.0, 20.0, (ncol, nlay)))}
    lo, hi = {1: (14.0, 125.0), 2: (6.0, 128.0), 3: (6.0, 135.0)}[iceflag]
    mc["reicmcl"] = np.asfortranarray(rng.uniform(lo, hi, (ncol, nlay)))
    return mc


# ---------------------------------------------------------------- tables
def test_reduced_tables_shapes_and_solar_source():
    t = _tables()
    assert list(t["ngc"]) == NGS and int(t["ngs"][-1]) == 112
    assert list(np.bincount(t["ngb"] - 16, minlength=14)) == NGS
    total = 0.0
    for k, b in enumerate(range(16, 30)):
        sf = np.asarray(t[f"b{b}.sfluxref"])
        assert sf.shape[0] == NGS[k]
        col = sf if sf.ndim == 1 else sf[:, 0]
        total += col.sum()
    # the Kurucz source of the reference (the bands with a binary-species
    # source hold one column per species ratio; the first column's totals)
    assert 1360.0 < total < 1375.0


def test_reduction_weights_are_convex():
    import os

    from brams_gb300.data.extract_sw_tables import reduction_weights

    t = _tables()
    rw = reduction_weights(t).reshape(14, 16)
    gs = 0
    for k in range(14):
        counts = t["ngn"][gs:gs + NGS[k]]
        gs += NGS[k]
        ipr = 0
        for n in counts:
            assert abs(rw[k, ipr:ipr + n].sum() - 1.0) < 1e-12
            ipr += n
        assert ipr == 16


# ---------------------------------------------------------------- oracle pins
def test_incoming_flux_is_the_solar_source():
    st = sw_state()
    o = pyoracle.rrtmg_sw(st, None, icld=0, iaer=0, scon=0.0, adjes=1.0)
    assert np.allclose(o["swdflx"][:, -1] / st["coszen"], 1368.22, atol=0.01)
    o2 = pyoracle.rrtmg_sw(st, None, icld=0, iaer=0, scon=0.0, dyofyr=3)  # near perihelion
    assert (o2["swdflx"][:, -1] > o["swdflx"][:, -1] * 1.03).all()
    o3 = pyoracle.rrtmg_sw(st, None, icld=0, iaer=0, scon=1361.0)
    assert np.allclose(o3["swdflx"][:, -1] / st["coszen"], 1361.0, atol=0.02)


def test_surface_reflects_its_albedo():
    st = sw_state()
    for k in ("asdir", "asdif", "aldir", "aldif"):
        st[k] = np.full_like(st[k], 0.3)
    o = pyoracle.rrtmg_sw(st, None, icld=0, iaer=0)
    assert np.allclose(o["swuflxc"][:, 0] / o["swdflxc"][:, 0], 0.3, rtol=1e-12)


def test_scattering_atmosphere_conserves_energy():
    st = sw_state(ncol=4)
    for k in ("h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr"):
        st[k] = np.zeros_like(st[k], order="F")
    o = pyoracle.rrtmg_sw(st, None, icld=0, iaer=0)
    net = o["swdflx"] - o["swuflx"]
    assert np.abs(net - net[:, -1:]).max() < 1e-6 * net.max()
    assert np.abs(o["swhr"]).max() < 1e-6


@pytest.mark.parametrize("scale,laytrop", [(1.0, None), (0.08, 0), (None, "all")])
def test_columns_wholly_above_or_below_the_tropopause_switch(scale, laytrop):
    """Columns whose layers all lie above (laytrop 0) or all below (laytrop =
    nlay) the lower/upper switch at log p = 4.56: the solar-layer searches of
    the bands take their other branch (the reference reads jp(0) or
    jp(nlayers+1) there, taken as 0).  Fluxes stay finite and the column
    absorbs (net flux falls downward).  The incoming flux is the solar source
    for a full column; a band whose solar-source layer the column never
    reaches gets none (the reference leaves its source unset; the
    restatement takes 0), so a squeezed column receives less."""
    st = sw_state(ncol=6, nlay=30, seed=44)
    if scale is None:  # squeeze the column between the surface and 200 hPa
        for k in ("play", "plev"):
            p = st[k]
            st[k] = np.asfortranarray(p[:, :1] - (p[:, :1] - p) * (p[:, :1] - 200.0) / (p[:, :1] - p[:, -1:]))
    elif scale != 1.0:
        for k in ("play", "plev"):
            st[k] = np.asfortranarray(st[k] * scale)
    lp = np.log(st["play"])
    if laytrop == 0:
        assert (lp <= 4.56).all()
    elif laytrop == "all":
        assert (lp > 4.56).all()
    o = pyoracle.rrtmg_sw(st, None, icld=0, iaer=10)
    for k in ("swuflx", "swdflx", "swhr"):
        assert np.isfinite(o[k]).all(), k
    net = o["swdflx"] - o["swuflx"]
    assert (net[:, -1] >= net[:, 0] - 1e-9).all()
    toa = o["swdflx"][:, -1] / st["coszen"]
    if scale == 1.0:
        assert np.allclose(toa, 1368.22, atol=0.01)
    else:
        assert (toa > 0.0).all() and (toa < 1368.22 - 1.0).all()


def test_clouds_add_reflection():
    st = sw_state(cloud_prob=0.8)
    mc = sw_mcica(st)
    o = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10)
    assert (o["swuflx"][:, -1] >= o["swuflxc"][:, -1] - 1e-9).all()
    assert (o["swuflx"][:, -1] - o["swuflxc"][:, -1]).max() > 10.0


# ---------------------------------------------------------------- GPU parity
TOL = {64: (1e-6, 1e-8), 32: (0.05, 0.01)}  # bits -> (W m-2, K/day)
BITS = [64, 32]


def _parity(out, ref, bits=64):
    flux_tol, hr_tol = TOL[bits]
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
        assert np.abs(out[k] - ref[k]).max() <= flux_tol, (k, float(np.abs(out[k] - ref[k]).max()))
    for k in ("swhr", "swhrc"):
        assert np.abs(out[k] - ref[k]).max() <= hr_tol, (k, float(np.abs(out[k] - ref[k]).max()))


@pytest.fixture(scope="module")
def swctx(ctx):
    ctx.sw_ini(1004.0)
    yield ctx
    ctx.sw_set_precision(32)


def _solve(swctx, bits, *args, **kw):
    swctx.sw_set_precision(bits)
    return swctx.rrtmg_sw(*args, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("bits", BITS)
@pytest.mark.parametrize("nlay", [38, 45, 60])
def test_clear_sky_matches_oracle(swctx, nlay, bits):
    st = sw_state(ncol=96, nlay=nlay, seed=nlay)
    st["coszen"][:3] = [1.0, 1e-3, -0.2]  # overhead, grazing and night
    for iaer in (0, 10):
        ref = pyoracle.rrtmg_sw(st, None, icld=0, iaer=iaer)
        out = _solve(swctx, bits, st, None, icld=0, iaer=iaer)
        _parity(out, ref, bits)


@pytest.mark.gpu
@pytest.mark.parametrize("bits", BITS)
@pytest.mark.parametrize("iceflag", [1, 2, 3])
def test_mcica_clouds_match_oracle(swctx, iceflag, bits):
    st = sw_state(ncol=128, nlay=45, seed=10 + iceflag, cloud_prob=0.7)
    mc = sw_mcica(st, seed=iceflag, iceflag=iceflag)
    ref = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10, iceflgsw=iceflag, dyofyr=172, scon=1361.0)
    out = _solve(swctx, bits, st, mc, icld=3, iaer=10, iceflgsw=iceflag, dyofyr=172, scon=1361.0)
    _parity(out, ref, bits)
    assert np.abs(out["swdflx"] - out["swdflxc"]).max() > 10.0


@pytest.mark.gpu
@pytest.mark.parametrize("bits", BITS)
def test_direct_cloud_optics_match_oracle(swctx, bits):
    """inflag 0: the caller's cloud optical depth, albedo, asymmetry and
    forward-scattering fraction, delta-scaled by cldprmc_sw."""
    st = sw_state(ncol=64, nlay=38, seed=77, cloud_prob=0.6)
    mc = sw_mcica(st, seed=5)
    ref = pyoracle.rrtmg_sw(st, mc, icld=2, iaer=0, inflgsw=0)
    out = _solve(swctx, bits, st, mc, icld=2, iaer=0, inflgsw=0)
    _parity(out, ref, bits)


@pytest.mark.gpu
@pytest.mark.parametrize("bits", BITS)
def test_device_entry_with_wide_leading_dimension(swctx, bits):
    import torch

    from brams_gb300 import rrtmg_lw as R

    st = sw_state(ncol=40, nlay=45, seed=91, cloud_prob=0.6)
    mc = sw_mcica(st, seed=9)
    ref = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10)
    ncol, nlay = st["play"].shape
    ld = 53
    dev = torch.device("cuda", 0)

    def dv(a, axis):  # Fortran array padded to leading dimension ld on `axis`, on the device
        a = np.asarray(a, dtype=np.float64)
        shape = list(a.shape)
        shape[axis] = ld
        w = np.zeros(shape, order="F")
        idx = [slice(None)] * a.ndim
        idx[axis] = slice(0, a.shape[axis])
        w[tuple(idx)] = a
        return torch.from_numpy(np.ascontiguousarray(w.T)).to(dev)

    d = {k: dv(st[k], 0) for k in R.SW_STATE}
    for k in ("tauaer_sw", "ssaaer_sw", "asmaer_sw"):
        d[k] = dv(st[k], 0)
    for k in R.SW_CLOUD:
        d[k] = dv(mc[k], 1 if mc[k].ndim == 3 else 0)
    outs = {k: torch.zeros((nlay + 1, ld), dtype=torch.float64, device=dev) for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    outs["swhr"] = torch.zeros((nlay, ld), dtype=torch.float64, device=dev)
    outs["swhrc"] = torch.zeros((nlay, ld), dtype=torch.float64, device=dev)
    status = torch.full((ncol,), -1, dtype=torch.int32, device=dev)
    import ctypes as C

    swctx.sw_set_precision(bits)
    ic, ia = C.c_int(3), C.c_int(10)
    args = [swctx.h, None, ncol, nlay, C.byref(ic), C.byref(ia)] + [d[k].data_ptr() for k in R.SW_STATE]
    args += [1.0, 0, 1368.22, -1, 2, 3, 1] + [d[k].data_ptr() for k in R.SW_CLOUD]
    args += [d["tauaer_sw"].data_ptr(), d["ssaaer_sw"].data_ptr(), d["asmaer_sw"].data_ptr(), None]
    args += [outs[k].data_ptr() for k in R.SW_OUT] + [ld, ld, status.data_ptr()]
    rc = swctx.L.gb_rrtmg_sw_device(*args)
    assert rc == 0
    torch.cuda.synchronize()
    assert (status.cpu().numpy() == 0).all()
    got = {k: v.cpu().numpy().T[:ncol] for k, v in outs.items()}
    _parity(got, ref, bits)


@pytest.mark.gpu
@pytest.mark.parametrize("bits", BITS)
def test_radius_bounds_are_decided_on_the_double_inputs(swctx, bits):
    """cldprmc_sw's stops (ice option 3: generalized effective size 5-140 um;
    liquid option 1: radius 2.5-60 um) on the double radii: a radius on a
    bound passes, one a rounding step beyond it stops the call, in both
    precisions (the fp32 kernel rounds both to the same float)."""
    from brams_gb300.rrtmg_lw import RrtmgLwError

    st = sw_state(ncol=8, nlay=20, seed=3, cloud_prob=1.0)
    mc = sw_mcica(st, seed=2)
    shape = mc["cldfmcl"].shape
    mc["cldfmcl"] = np.asfortranarray(np.ones(shape))
    mc["ciwpmcl"] = np.asfortranarray(np.full(shape, 5.0))
    mc["clwpmcl"] = np.asfortranarray(np.full(shape, 8.0))
    for key, edge, code in (("reicmcl", 140.0, 5), ("reicmcl", 5.0, 5), ("relqmcl", 60.0, 6), ("relqmcl", 2.5, 6)):
        ok = {k: np.array(v, order="F") for k, v in mc.items()}
        ok[key][3, 7] = edge
        ref = pyoracle.rrtmg_sw(st, ok, icld=3, iaer=10)
        _parity(_solve(swctx, bits, st, ok, icld=3, iaer=10), ref, bits)
        beyond = np.nextafter(edge, np.inf if edge > 10.0 else -np.inf)
        assert np.float32(beyond) == np.float32(edge)
        bad = {k: np.array(v, order="F") for k, v in ok.items()}
        bad[key][3, 7] = beyond
        with pytest.raises(RrtmgLwError) as e:
            _solve(swctx, bits, st, bad, icld=3, iaer=10)
        assert e.value.code == code, (key, edge)


# ---------------------------------------------------------------- cldprop_sw (oracle)
def test_oracle_cldprop_sw_clear_layers_and_direct_input():
    """Clear layers keep (taucldorig = tauc, 0, 1, 0); with direct input
    (inflag 0) the band values are the delta scaling of rrtmg_sw_cldprop.f90:
    161-176 of the inputs."""
    st = make_state(ProfileSpec(ncol=5, nlay=20, seed=8, cloud_prob=0.6))
    rng = np.random.default_rng(8)
    bi = {"tauc": rng.uniform(0.1, 5.0, (14, 5, 20)), "ssac": rng.uniform(0.8, 0.999, (14, 5, 20)),
          "asmc": rng.uniform(0.6, 0.9, (14, 5, 20)), "fsfc": rng.uniform(0.0, 0.4, (14, 5, 20))}
    o, status = pyoracle.cldprop_sw_columns(st, bi, inflag=0)
    assert (status == 0).all()
    cloudy = (st["cldfrac"] >= 1e-20)[None].repeat(14, 0)  # tauc > 0 everywhere, so the cloud fraction decides
    assert cloudy.any() and (~cloudy).any()
    f, w, t, g = bi["fsfc"], bi["ssac"], bi["tauc"], bi["asmc"]
    assert np.array_equal(o["taucloud"][cloudy], ((1.0 - f * w) * t)[cloudy])
    assert np.array_equal(o["ssacloud"][cloudy], ((1.0 - f) * w / (1.0 - f * w))[cloudy])
    assert np.array_equal(o["asmcloud"][cloudy], ((g - f) / (1.0 - f))[cloudy])
    assert np.array_equal(o["taucldorig"], t)
    for k, v in (("taucloud", 0.0), ("ssacloud", 1.0), ("asmcloud", 0.0)):
        assert (o[k][~cloudy] == v).all(), k


@pytest.mark.parametrize("iceflag", [1, 2, 3])
def test_oracle_cldprop_sw_water_paths(iceflag):
    """Optics from water paths (inflag 2): delta scaling only lowers the
    optical depth, albedos in (0, 1], asymmetries in [0, 1); the band values
    feed mcica_subcol_sw in its (14, ncol, nlay) layout."""
    st = make_state(ProfileSpec(ncol=6, nlay=30, seed=20 + iceflag, cloud_prob=0.7))
    rng = np.random.default_rng(iceflag)
    lo, hi = {1: (13.0, 130.0), 2: (5.0, 131.0), 3: (5.0, 140.0)}[iceflag]
    st["rei"] = np.asfortranarray(rng.uniform(lo, hi, st["rei"].shape))
    st["rel"] = np.asfortranarray(rng.uniform(2.5, 60.0, st["rel"].shape))
    o, status = pyoracle.cldprop_sw_columns(st, iceflag=iceflag)
    assert (status == 0).all()
    cl = o["taucloud"] > 0
    assert cl.any()
    assert (o["taucloud"][cl] <= o["taucldorig"][cl] * (1 + 1e-12)).all()
    assert (o["ssacloud"][cl] > 0).all() and (o["ssacloud"][cl] <= 1.0).all()
    assert (o["asmcloud"][cl] >= 0).all() and (o["asmcloud"][cl] < 1.0).all()
    band = {"tauc": o["taucloud"], "ssac": o["ssacloud"], "asmc": o["asmcloud"], "fsfc": np.zeros_like(o["taucloud"])}
    mc = pyoracle.mcica_subcol_sw(st, band, 3, 9)
    ngb = np.repeat(np.arange(14), NGS)
    cloudy = mc["cldfmcl"] == 1.0
    assert np.array_equal(mc["taucmcl"][cloudy], o["taucloud"][ngb][cloudy])


@pytest.mark.parametrize("inflag,iceflag", [(2, 1), (2, 2), (2, 3), (0, 3)])
def test_the_two_cloud_optics_restatements_agree(inflag, iceflag):
    """cldprop_sw (rrtmg_sw_cldprop.f90, per band and layer) and cldprmc_sw
    (rrtmg_sw_cldprmc.f90, per g-point and layer), restated from two
    reference files, give every overcast g-point exactly its band's values."""
    import ctypes as C

    ncol, nlay = 4, 24
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=30 + iceflag, cloud_prob=0.7))
    rng = np.random.default_rng(iceflag)
    lo, hi = {1: (13.0, 130.0), 2: (5.0, 131.0), 3: (5.0, 140.0)}[iceflag]
    st["rei"] = np.asfortranarray(rng.uniform(lo, hi, (ncol, nlay)))
    st["rel"] = np.asfortranarray(rng.uniform(2.5, 60.0, (ncol, nlay)))
    bi = {"tauc": rng.uniform(0.1, 5.0, (14, ncol, nlay)), "ssac": rng.uniform(0.8, 0.999, (14, ncol, nlay)),
          "asmc": rng.uniform(0.6, 0.9, (14, ncol, nlay)), "fsfc": rng.uniform(0.0, 0.4, (14, ncol, nlay))}
    band, status = pyoracle.cldprop_sw_columns(st, bi if inflag == 0 else None, inflag, iceflag, 1)
    assert (status == 0).all()
    L = pyoracle.sw_lib()
    ngb = np.repeat(np.arange(14), NGS)
    p = pyoracle._p
    for i in range(ncol):
        over = (st["cldfrac"][i] >= 1e-20).astype(np.float64)
        g_in = lambda a: np.asfortranarray(np.broadcast_to(a, (112, nlay)), dtype=np.float64)  # noqa: E731
        cm = {"cldfmc": g_in(over), "ciwpmc": g_in(st["ciwp"][i] * over), "clwpmc": g_in(st["clwp"][i] * over)}
        for k in ("tauc", "ssac", "asmc", "fsfc"):
            cm[k + "mc"] = g_in(bi[k][ngb, i, :] if inflag == 0 else np.zeros((112, nlay)))
        outs = [np.zeros((112, nlay), order="F") for _ in range(4)]
        rc = L.ora_cldprmc_sw_column(C.c_int(nlay), C.c_int(inflag), C.c_int(iceflag), C.c_int(1),
                                     *[p(cm[k]) for k in ("cldfmc", "taucmc", "ssacmc", "asmcmc", "fsfcmc",
                                                          "ciwpmc", "clwpmc")],
                                     p(np.ascontiguousarray(st["rei"][i])), p(np.ascontiguousarray(st["rel"][i])),
                                     *[p(o) for o in outs])
        assert rc == 0
        cloudy = over.astype(bool)
        assert cloudy.any()
        for o, k in zip(outs, ("taucldorig", "taucloud", "ssacloud", "asmcloud")):
            assert np.array_equal(o[:, cloudy], band[k][ngb, i][:, cloudy]), k


def test_oracle_cldprop_sw_stops_on_a_radius_out_of_bounds():
    st = make_state(ProfileSpec(ncol=3, nlay=12, seed=5, cloud_prob=1.0))
    st["rei"] = np.asfortranarray(np.full(st["rei"].shape, 150.0))
    _, status = pyoracle.cldprop_sw_columns(st, iceflag=3)
    icy = ((st["cldfrac"] >= 1e-20) & (st["ciwp"] > 0)).any(axis=1)
    assert (status[icy] == 5).all() and (status[~icy] == 0).all()  # 'ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS'


# ---------------------------------------------------------------- McICA for the shortwave
def _sw_band(st, seed=3):
    ncol, nlay = st["play"].shape
    rng = np.random.default_rng(seed)
    return {"tauc": np.asfortranarray(rng.uniform(0.1, 10.0, (14, ncol, nlay))),
            "ssac": np.asfortranarray(rng.uniform(0.8, 1.0, (14, ncol, nlay))),
            "asmc": np.asfortranarray(rng.uniform(0.6, 0.9, (14, ncol, nlay))),
            "fsfc": np.asfortranarray(rng.uniform(0.0, 0.5, (14, ncol, nlay)))}


def test_oracle_sw_mcica_maps_bands_and_clear_cells():
    st = make_state(ProfileSpec(ncol=6, nlay=20, seed=4, cloud_prob=0.7))
    band = _sw_band(st)
    o = pyoracle.mcica_subcol_sw(st, band, 3, 11)
    cloudy = o["cldfmcl"] == 1.0
    assert cloudy.any() and (~cloudy).any()
    assert (o["ssacmcl"][~cloudy] == 1.0).all() and (o["asmcmcl"][~cloudy] == 0.0).all()
    ngb = np.repeat(np.arange(14), NGS)  # sub-column -> band (0-based)
    for k, src in (("taucmcl", "tauc"), ("ssacmcl", "ssac"), ("fsfcmcl", "fsfc")):
        want = np.where(cloudy, band[src][ngb], o[k])
        assert np.array_equal(o[k], want), k


@pytest.mark.gpu
@pytest.mark.parametrize("icld", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("irng", [0, 1])
def test_sw_mcica_is_bit_exact(swctx, icld, irng):
    st = make_state(ProfileSpec(ncol=24, nlay=30, seed=40 + icld, cloud_prob=0.6))
    st["alpha"] = np.asfortranarray(np.exp(-np.linspace(0.1, 2.0, 30))[None, :] * np.ones((24, 1)))
    band = _sw_band(st, seed=icld)
    ref = pyoracle.mcica_subcol_sw(st, band, icld, 17, irng)
    got = swctx.mcica_subcol_sw(st, band, icld, 17, irng)
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.gpu
def test_sw_mcica_seed_per_column(swctx):
    """Per-column seeding: column c is the reference called alone with seed base + c."""
    st = make_state(ProfileSpec(ncol=12, nlay=25, seed=9, cloud_prob=0.6))
    band = _sw_band(st)
    got = swctx.mcica_subcol_sw(st, band, 3, 100, 1, seed_per_column=True)
    for c in range(12):
        sub = {k: np.asfortranarray(st[k][c:c + 1]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")}
        sb = {k: np.asfortranarray(v[:, c:c + 1]) for k, v in band.items()}
        ref = pyoracle.mcica_subcol_sw(sub, sb, 3, 100 + c, 1)
        for k in ("cldfmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl"):
            assert np.array_equal(got[k][:, c], ref[k][:, 0]), (c, k)


@pytest.mark.gpu
@pytest.mark.parametrize("bits", BITS)
def test_sw_chain_mcica_then_solver_matches_oracle(swctx, bits):
    """BRAMS's order: mcica_subcol_sw, then rrtmg_sw, both on the GPU."""
    st = sw_state(ncol=64, nlay=45, seed=31, cloud_prob=0.7)
    for k in ("rei", "rel"):
        st[k] = np.asfortranarray(np.clip(st[k], 6.0, 50.0))
    band = _sw_band(st, seed=8)
    mc_ref = pyoracle.mcica_subcol_sw(st, band, 3, 5)
    mc = swctx.mcica_subcol_sw(st, band, 3, 5)
    for k in mc_ref:
        assert np.array_equal(mc[k], mc_ref[k]), k
    ref = pyoracle.rrtmg_sw(st, mc_ref, icld=3, iaer=10)
    out = _solve(swctx, bits, st, mc, icld=3, iaer=10)
    _parity(out, ref, bits)
