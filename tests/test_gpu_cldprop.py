"""cldprop on the device (gb_cldprop_lw_device) against the oracle's
restatement of rrtmg_lw_cldprop.f90:50-295, column by column, for every
input option; its status codes; and the fused-cloud solver fed by it."""
import ctypes as C

import numpy as np
import pytest

import pyoracle
from brams_gb300 import rrtmg_lw as R
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu

# radius ranges each ice option accepts (the reference STOPs outside)
ICE_RANGE = {0: (10.0, 140.0), 1: (13.0, 130.0), 2: (5.0, 131.0), 3: (5.0, 140.0)}


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda()


def _state(ncol, nlay, seed, iceflag):
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=4.0, h2o_sigma=0.5))
    rs = np.random.default_rng(seed)
    lo, hi = ICE_RANGE[iceflag]
    st["rei"] = np.asfortranarray(rs.uniform(lo, hi, st["rei"].shape))
    st["rel"] = np.asfortranarray(rs.uniform(2.5, 60.0, st["rel"].shape))
    st["tauc_in"] = np.asfortranarray(rs.uniform(0.0, 2.0, (16,) + st["rei"].shape) * (rs.random((16,) + st["rei"].shape) < 0.3))
    return st


def _oracle(st, inflag, iceflag, liqflag):
    """Per column through ora_cldprop with the same tauc input; (16, ncol, nlay) and the status per column."""
    L = pyoracle.lib()
    ncol, nlay = st["cldfrac"].shape
    out = np.zeros((16, ncol, nlay), order="F")
    status = np.zeros(ncol, dtype=np.int64)
    tc = np.zeros((nlay, 16), order="F")
    nb = C.c_int(0)
    p = pyoracle._p
    for i in range(ncol):
        args = [np.ascontiguousarray(st[k][i, :]) for k in ("cldfrac",)]
        tin = np.asfortranarray(st["tauc_in"][:, i, :])
        rc = L.ora_cldprop(C.c_int(nlay), C.c_int(inflag), C.c_int(iceflag), C.c_int(liqflag),
                           p(args[0]), p(tin), p(np.ascontiguousarray(st["ciwp"][i, :])),
                           p(np.ascontiguousarray(st["clwp"][i, :])), p(np.ascontiguousarray(st["rei"][i, :])),
                           p(np.ascontiguousarray(st["rel"][i, :])), C.byref(nb), p(tc))
        status[i] = rc
        if rc == 0:
            out[:, i, :] = tc.T
    return out, status


def _device(ctx, st, inflag, iceflag, liqflag):
    import torch

    ncol, nlay = st["cldfrac"].shape
    d = {k: _dev(st[k]) for k in ("cldfrac", "ciwp", "clwp", "rei", "rel")}
    d["tauc"] = _dev(st["tauc_in"])
    d["taucloud"] = torch.full((nlay, ncol, 16), -1.0, dtype=torch.float64, device="cuda")
    d["d_col_status"] = torch.full((ncol,), -1, dtype=torch.int32, device="cuda")
    ctx.cldprop_lw_device(ncol, nlay, d, inflag, iceflag, liqflag)
    torch.cuda.synchronize()
    return d["taucloud"].cpu().numpy().T.copy(), d["d_col_status"].cpu().numpy()


@pytest.mark.parametrize("inflag,iceflag,liqflag", [(2, 3, 1), (2, 3, 0), (2, 2, 1), (2, 1, 1), (2, 1, 0),
                                                     (2, 0, 1), (2, 0, 0), (1, 3, 1), (0, 3, 1)])
def test_cldprop_matches_oracle(ctx, inflag, iceflag, liqflag):
    st = _state(97, 45, 200 + 10 * iceflag + liqflag, iceflag)
    ref, rs = _oracle(st, inflag, iceflag, liqflag)
    got, gs = _device(ctx, st, inflag, iceflag, liqflag)
    assert (rs == 0).all() and (gs == 0).all()
    assert ctx.sync_status() == 0
    scale = np.abs(ref).max() + 1e-300
    assert np.abs(got - ref).max() <= 1e-13 * scale, float(np.abs(got - ref).max())
    assert (got[ref == 0.0] == 0.0).all()  # bands a layer does not fill stay 0


def test_cldprop_status_of_a_radius_out_of_bounds(ctx):
    st = _state(40, 30, 7, 3)
    cloudy = (st["cldfrac"] >= 1e-20) & (st["ciwp"] > 0)
    i, lay = [int(v[0]) for v in np.nonzero(cloudy)]  # the first cloudy icy cell
    st["rei"][i, lay] = 200.0
    ref, rs = _oracle(st, 2, 3, 1)
    got, gs = _device(ctx, st, 2, 3, 1)
    assert rs[i] == 5 and gs[i] == 5  # 'ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS'
    ok = np.arange(40) != i
    assert (gs[ok] == 0).all()
    assert np.abs(got[:, ok, :] - ref[:, ok, :]).max() <= 1e-13 * np.abs(ref).max()
    assert ctx.sync_status() == 5


def test_fused_solver_fed_by_device_cldprop(ctx):
    """The fused-cloud batch with tauc from the device cldprop gives exactly
    what it gives with the oracle's tauc (BRAMS options)."""
    import torch

    st = make_state(ProfileSpec(ncol=64, nlay=45, seed=301, t_noise=4.0, h2o_sigma=0.5))
    tauc_ref = pyoracle.cldprop_columns(st)
    st["tauc_in"] = np.zeros((16,) + st["rei"].shape, order="F")
    tauc_dev, _ = _device(ctx, st, 2, 3, 1)
    assert np.abs(tauc_dev - tauc_ref).max() <= 1e-13 * np.abs(tauc_ref).max()
    from brams_gb300 import surrogate as S

    ga, gb = S.DeviceGrid(st, tauc_ref), S.DeviceGrid(st, tauc_dev)
    ctx.rrtmg_lw_batch_device([ga.desc(seed0=11), gb.desc(seed0=11)])
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    a, b = ga.outputs(), gb.outputs()
    for k in a:
        assert np.abs(a[k] - b[k]).max() <= 1e-9 * (np.abs(a[k]).max() + 1.0), k


@pytest.mark.parametrize("inflag,iceflag,liqflag", [(2, 3, 1), (2, 1, 0), (0, 3, 1)])
def test_output_off_16_byte_boundary_gives_the_same_bits(ctx, inflag, iceflag, liqflag):
    """An output array that starts 8 bytes past a 16-byte boundary takes the
    kernel's one-value-at-a-time stores instead of its pairs: same values."""
    import torch

    st = _state(61, 45, 300 + 10 * iceflag + liqflag, iceflag)
    ncol, nlay = st["cldfrac"].shape
    a, _ = _device(ctx, st, inflag, iceflag, liqflag)
    d = {k: _dev(st[k]) for k in ("cldfrac", "ciwp", "clwp", "rei", "rel")}
    d["tauc"] = _dev(st["tauc_in"])
    flat = torch.full((nlay * ncol * 16 + 1,), -1.0, dtype=torch.float64, device="cuda")
    d["taucloud"] = flat[1:].view(nlay, ncol, 16)
    assert d["taucloud"].data_ptr() % 16 == 8
    ctx.cldprop_lw_device(ncol, nlay, d, inflag, iceflag, liqflag)
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    b = d["taucloud"].cpu().numpy().T.copy()
    assert np.array_equal(a, b)
    assert flat[0].item() == -1.0  # nothing written before the array
