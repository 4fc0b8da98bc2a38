"""BRAMS's column packing and tendency write-back on the device
(gb_rtm_pack_lw_device / gb_rtm_unpack_lw_device, and the shortwave-only
gb_rtm_pack_sw_device / gb_rtm_unpack_sw_device) against the CPU
restatement (oracle/brams_pack.py), and the whole caller-side path: model
state in, packed on the device, cldprop and the fused-cloud solver, theta
tendency out, against the same chain on the FP64 oracle."""
import os
import sys

import numpy as np
import pytest

from brams_fields import brams_fields, ozone
from brams_gb300 import rrtmg_lw as R

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import brams_pack as BP  # noqa: E402

pytestmark = pytest.mark.gpu

# values that go through a real(8) power (pressures, the top interface
# temperature extrapolated in pressure, the surface temperature): CUDA's pow
# and the host's may differ in the last bits
POW = ("play", "plev", "tlev", "tsfc")


def _upload(f):
    import torch

    return {k: torch.from_numpy(np.ascontiguousarray(v.T)).cuda() for k, v in f.items()}  # memory order = Fortran


def _pack_device(ctx, f, box, iceflgsw, firsttime, ld=None):
    import torch

    mzp, mxp, myp = f["pi0"].shape
    ia, iz, ja, jz = box
    ncol, nlay = (iz - ia + 1) * (jz - ja + 1), mzp - 1
    ld = ld or ncol
    d = _upload(f)
    shapes = {"plev": nlay + 1, "tlev": nlay + 1, "tsfc": 1, "emis": 16}
    for k in R.Context.PACK_OUT:
        d[k] = torch.full((shapes.get(k, nlay), ld), -7.0, dtype=torch.float64, device="cuda")
    ctx.rtm_pack_lw_device(mzp, mxp, myp, box, d, iceflgsw=iceflgsw, firsttime=firsttime, ld=ld)
    torch.cuda.synchronize()
    return d, ncol, nlay


@pytest.mark.parametrize("box,iceflgsw,firsttime,ld", [((1, 9, 1, 7), 3, False, None), ((2, 8, 3, 7), 1, False, 40),
                                                       ((3, 3, 2, 6), 2, True, None), ((1, 9, 1, 7), 0, False, None)])
def test_pack_matches_oracle(ctx, box, iceflgsw, firsttime, ld):
    f = brams_fields(33, 9, 7, seed=21 + iceflgsw)
    ref = BP.pack_lw(f, *box, iceflgsw=iceflgsw, firsttime=firsttime)
    d, ncol, nlay = _pack_device(ctx, f, box, iceflgsw, firsttime, ld)
    assert ctx.sync_status() == 0
    names = {"reic": "rei", "relq": "rel"}
    for k in R.Context.PACK_OUT:
        got = d[k].cpu().numpy().T[:ncol]  # (ncol, levels)
        want = ref[names.get(k, k)].reshape(ncol, -1)
        if k in POW:
            assert np.allclose(got, want, rtol=1e-14, atol=0.0), (k, float(np.abs(got - want).max()))
        else:
            assert np.array_equal(got, want), k
        if ld:
            assert (d[k].cpu().numpy().T[ncol:] == -7.0).all(), k  # rows past the columns stay untouched


def test_unpack_matches_oracle(ctx):
    import torch

    mzp, mxp, myp, box = 12, 6, 5, (2, 5, 2, 4)
    ncol = 12
    rs = np.random.default_rng(9)
    hr = rs.normal(0.0, 3.0, (ncol + 3, mzp - 1))  # leading dimension 15 > ncol
    sw = rs.normal(0.0, 2.0, (ncol + 3, mzp - 1))
    dflx = rs.uniform(150.0, 450.0, (ncol + 1, mzp))
    f0 = np.full((mzp, mxp, myp), 5.0, np.float32)
    r0 = np.full((mxp, myp), 4.0, np.float32)
    for swhr in (None, sw):
        ref_f, ref_r = BP.unpack_lw(hr[:ncol], dflx[:ncol], None if swhr is None else swhr[:ncol],
                                    mzp, mxp, myp, *box, f0, r0)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
        fth, rl = dev(f0), dev(r0)
        ctx.rtm_unpack_lw_device(mzp, mxp, myp, box, dev(hr), dev(dflx), fth, rl,
                                 swhr=None if swhr is None else dev(swhr), ld_hr=ncol + 3, ld_flx=ncol + 1)
        torch.cuda.synchronize()
        assert np.array_equal(fth.cpu().numpy().T, ref_f)
        assert np.array_equal(rl.cpu().numpy().T, ref_r)
    assert ctx.sync_status() == 0


def test_model_state_in_theta_tendency_out(ctx):
    """BRAMS fields -> packed columns -> cldprop -> fused McICA solver ->
    theta tendency and surface flux, all on the device, against the oracle
    chain (packing restatement, cldprop, McICA with seed = base + column,
    FP64 rrtmg_lw, write-back) within the solver's parity tolerances."""
    import pyoracle
    import torch

    mzp, mxp, myp, box, seed0 = 41, 12, 10, (2, 11, 2, 9), 77
    f = brams_fields(mzp, mxp, myp, seed=5)
    d, ncol, nlay = _pack_device(ctx, f, box, 3, False)
    ref = BP.pack_lw(f, *box, iceflgsw=3)
    o3 = ozone(ref["play"])
    d["o3vmr"] = torch.from_numpy(np.ascontiguousarray(o3.T)).cuda()
    d["tauaer"] = torch.zeros((16, nlay, ncol), dtype=torch.float64, device="cuda")
    d["tauc"] = torch.empty((nlay, ncol, 16), dtype=torch.float64, device="cuda")
    for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
        d[k] = torch.empty((nlay + 1, ncol), dtype=torch.float64, device="cuda")
    d["hr"] = torch.empty((nlay, ncol), dtype=torch.float64, device="cuda")
    d["hrc"] = torch.empty((nlay, ncol), dtype=torch.float64, device="cuda")
    ctx.cldprop_lw_device(ncol, nlay, {"cldfrac": d["cldfrac"], "ciwp": d["ciwp"], "clwp": d["clwp"],
                                       "rei": d["reic"], "rel": d["relq"], "taucloud": d["tauc"]})
    arrays = dict(d)
    arrays["reicmcl"], arrays["relqmcl"] = d["reic"], d["relq"]
    ctx.rrtmg_lw_batch_device([R.grid_desc(ncol, nlay, arrays, icld=3, cloud_mode=R.CLOUD_FUSED, seed0=seed0)])
    fth = torch.zeros((myp, mxp, mzp), dtype=torch.float32, device="cuda")
    rl = torch.zeros((myp, mxp), dtype=torch.float32, device="cuda")
    ctx.rtm_unpack_lw_device(mzp, mxp, myp, box, d["hr"], d["dflx"], fth, rl, ld_flx=ncol)
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    st = {k: np.asfortranarray(v) for k, v in ref.items()}
    st["o3vmr"] = o3
    st["tauaer"] = np.zeros((ncol, nlay, 16), order="F")
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=seed0)
    out = pyoracle.rrtmg_lw(st, mc, icld=3)
    ref_f, ref_r = BP.unpack_lw(out["hr"], out["dflx"], None, mzp, mxp, myp, *box)
    got_f, got_r = fth.cpu().numpy().T, rl.cpu().numpy().T
    assert np.abs(got_f - ref_f).max() <= 0.01 / 86400.0, float(np.abs(got_f - ref_f).max() * 86400.0)
    assert np.abs(got_r - ref_r).max() <= 0.05
    assert np.abs(ref_f).max() > 1e-6  # the tendency is not trivially zero


@pytest.mark.parametrize("firsttime", [False, True])
def test_shortwave_pack_and_unpack_match_oracle(ctx, firsttime):
    import torch

    mxp, myp, box = 9, 7, (2, 8, 3, 7)
    rs = np.random.default_rng(17)
    cosz = rs.uniform(-0.3, 1.0, (mxp, myp)).astype(np.float32)
    albedt = rs.uniform(0.05, 0.6, (mxp, myp)).astype(np.float32)
    ref = BP.pack_sw(cosz, albedt, *box, firsttime=firsttime)
    ncol = ref["coszen"].size
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # noqa: E731
    out = {k: torch.full((ncol,), -7.0, dtype=torch.float64, device="cuda") for k in ref}
    ctx.rtm_pack_sw_device(mxp, myp, box, dev(cosz), dev(albedt), out, firsttime=firsttime)
    swdflx = rs.uniform(0.0, 900.0, (ncol + 2, 4))
    swdflx[::5, 0] = rs.uniform(0.0, 0.6, swdflx[::5, 0].shape)  # fluxes around the 0.5 W m-2 cut
    r0 = np.full((mxp, myp), 2.0, np.float32)
    want = BP.unpack_sw(swdflx[:ncol], mxp, myp, *box, r0)
    rsh = dev(r0)
    ctx.rtm_unpack_sw_device(mxp, myp, box, dev(swdflx[:, 0].copy()), rsh)
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    for k in ref:
        assert np.array_equal(out[k].cpu().numpy(), ref[k]), k
    assert np.array_equal(rsh.cpu().numpy().T, want)
