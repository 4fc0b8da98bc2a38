"""cldprop_sw on the device (gb_cldprop_sw_device) against the oracle's
restatement of rrtmg_sw_cldprop.f90:53-365, column by column, for the input
options; its status codes; and BRAMS's shortwave cloud chain on the device
(cldprop_sw, then mcica_subcol_sw, then rrtmg_sw) against the oracle's."""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu

ICE_RANGE = {1: (13.0, 130.0), 2: (5.0, 131.0), 3: (5.0, 140.0)}
OUTS = ("taucloud", "ssacloud", "asmcloud", "taucldorig")


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda()


def _state(ncol, nlay, seed, iceflag):
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=4.0, h2o_sigma=0.5, cloud_prob=0.7))
    rs = np.random.default_rng(seed)
    lo, hi = ICE_RANGE[iceflag]
    st["rei"] = np.asfortranarray(rs.uniform(lo, hi, st["rei"].shape))
    st["rel"] = np.asfortranarray(rs.uniform(2.5, 60.0, st["rel"].shape))
    shp = (14,) + st["rei"].shape
    band = {"tauc": rs.uniform(0.0, 3.0, shp) * (rs.random(shp) < 0.5), "ssac": rs.uniform(0.8, 0.999, shp),
            "asmc": rs.uniform(0.6, 0.9, shp), "fsfc": rs.uniform(0.0, 0.4, shp)}
    return st, {k: np.asfortranarray(v) for k, v in band.items()}


def _device(ctx, st, band, inflag, iceflag, liqflag):
    import torch

    ncol, nlay = st["cldfrac"].shape
    d = {k: _dev(st[k]) for k in ("cldfrac", "ciwp", "clwp", "rei", "rel")}
    if band is not None:
        d.update({k: _dev(v) for k, v in band.items()})
    for k in OUTS:
        d[k] = torch.full((nlay, ncol, 14), -7.0, dtype=torch.float64, device="cuda")
    d["d_col_status"] = torch.full((ncol,), -1, dtype=torch.int32, device="cuda")
    ctx.cldprop_sw_device(ncol, nlay, d, inflag, iceflag, liqflag)
    torch.cuda.synchronize()
    return {k: d[k].cpu().numpy().T.copy() for k in OUTS}, d["d_col_status"].cpu().numpy()


@pytest.fixture(scope="module")
def swctx(ctx):
    ctx.sw_ini(1004.0)
    return ctx


@pytest.mark.parametrize("inflag,iceflag,liqflag", [(2, 3, 1), (2, 2, 1), (2, 1, 1), (0, 3, 1), (1, 3, 1)])
@pytest.mark.parametrize("with_band", [True, False])
def test_cldprop_sw_matches_oracle(swctx, inflag, iceflag, liqflag, with_band):
    if inflag == 0 and not with_band:
        pytest.skip("direct input needs the band arrays")
    st, band = _state(83, 45, 400 + 10 * iceflag + inflag, iceflag)
    band = band if with_band else None
    ref, rs = pyoracle.cldprop_sw_columns(st, band, inflag, iceflag, liqflag)
    got, gs = _device(swctx, st, band, inflag, iceflag, liqflag)
    assert (rs == 0).all() and (gs == 0).all()
    assert swctx.sync_status() == 0
    for k in OUTS:
        scale = np.abs(ref[k]).max() + 1e-300
        assert np.abs(got[k] - ref[k]).max() <= 1e-13 * scale, (k, float(np.abs(got[k] - ref[k]).max()))
    if inflag != 1:
        assert (ref["taucloud"] > 0).mean() > 0.1


def test_cldprop_sw_status_of_a_radius_out_of_bounds(swctx):
    st, _ = _state(40, 30, 7, 3)
    cloudy = (st["cldfrac"] >= 1e-20) & (st["ciwp"] > 0)
    i, lay = [int(v[0]) for v in np.nonzero(cloudy)]  # the first cloudy icy cell
    st["rei"][i, lay] = 200.0
    ref, rs = pyoracle.cldprop_sw_columns(st, None, 2, 3, 1)
    got, gs = _device(swctx, st, None, 2, 3, 1)
    assert rs[i] == 5 and gs[i] == 5  # 'ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS'
    ok = np.arange(40) != i
    assert (gs[ok] == 0).all()
    for k in OUTS:
        assert np.abs(got[k][:, ok, :] - ref[k][:, ok, :]).max() <= 1e-13 * (np.abs(ref[k]).max() + 1e-300), k
    # the offending layer keeps the clear values
    assert (got["taucloud"][:, i, lay] == 0.0).all() and (got["ssacloud"][:, i, lay] == 1.0).all()
    assert (got["asmcloud"][:, i, lay] == 0.0).all()
    assert swctx.sync_status() == 5


def test_shortwave_cloud_chain_on_the_device(swctx):
    """BRAMS's order with the band optics from the device cldprop_sw: the
    McICA draws equal the oracle's bit for bit and the fluxes match the
    oracle's chain (fp64 kernel)."""
    st, _ = _state(48, 45, 21, 3)
    rs = np.random.default_rng(21)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        st[k] = rs.uniform(0.05, 0.6, 48)
    st["coszen"] = rs.uniform(0.1, 1.0, 48)
    ref_band, rstat = pyoracle.cldprop_sw_columns(st)
    got_band, gstat = _device(swctx, st, None, 2, 3, 1)
    assert (rstat == 0).all() and (gstat == 0).all()
    tobands = lambda o: {"tauc": o["taucloud"], "ssac": o["ssacloud"], "asmc": o["asmcloud"],  # noqa: E731
                         "fsfc": np.zeros_like(o["taucloud"])}
    mc_ref = pyoracle.mcica_subcol_sw(st, tobands(ref_band), 3, 13)
    mc = swctx.mcica_subcol_sw(st, tobands(got_band), 3, 13)
    assert np.array_equal(mc["cldfmcl"], mc_ref["cldfmcl"])
    for k in ("taucmcl", "ssacmcl", "asmcmcl"):
        assert np.abs(mc[k] - mc_ref[k]).max() <= 1e-13 * np.abs(mc_ref[k]).max(), k
    ref = pyoracle.rrtmg_sw(st, mc_ref, icld=3, iaer=0)
    swctx.sw_set_precision(64)
    try:
        out = swctx.rrtmg_sw(st, mc, icld=3, iaer=0)
    finally:
        swctx.sw_set_precision(32)
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
        assert np.abs(out[k] - ref[k]).max() <= 1e-6, k
    for k in ("swhr", "swhrc"):
        assert np.abs(out[k] - ref[k]).max() <= 1e-8, k
