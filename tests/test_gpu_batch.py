"""Batched grids in one persistent launch, in-kernel McICA, kernel variants,
CUDA-graph replay and the autotuner -- all through the C ABI.

Every batched result must be bit-identical to the single-grid entry point:
the batch only changes which block solves which column, and each column is
solved by the same code in the same order whatever the launch shape.  The
fused-cloud mode must equal mcica_subcol_lw (icld 3, Mersenne twister, seed
base + column) followed by rrtmg_lw, bit for bit.
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300 import rrtmg_lw as R
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu

FLUX_TOL = 0.05
HR_TOL = 0.01
OUTS = ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt")
GRIDS = [(37, 45, 101), (20, 38, 102), (13, 60, 103)]  # (ncol, nlay, seed)


def _dev(a):
    import torch

    # a Fortran-ordered array's memory is the C order of its transpose
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda()


class Grid:
    """One grid's inputs on the device, in both cloud modes."""

    def __init__(self, ncol, nlay, seed, seed0, tnoise=4.0):
        import torch

        spec = ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=tnoise)
        self.st = make_state(spec)
        self.tauc = pyoracle.cldprop_columns(self.st)
        self.ncol, self.nlay, self.seed0 = ncol, nlay, seed0
        d = {k: _dev(self.st[k]) for k in R.STATE_ORDER}
        d["tauaer"] = _dev(self.st["tauaer"])
        for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
            d[k] = _dev(self.st[k])
        d["tauc"] = _dev(self.tauc)
        for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl"):
            d[k] = torch.zeros((nlay, ncol, 140), dtype=torch.float64, device="cuda")
        d["reicmcl"] = torch.zeros((nlay, ncol), dtype=torch.float64, device="cuda")
        d["relqmcl"] = torch.zeros((nlay, ncol), dtype=torch.float64, device="cuda")
        self.d = d
        self.out = self.new_out()

    def new_out(self):
        import torch

        o = {k: torch.full((self.nlay + 1, self.ncol), -1.0, dtype=torch.float64, device="cuda")
             for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
        o["hr"] = torch.full((self.nlay, self.ncol), -1.0, dtype=torch.float64, device="cuda")
        o["hrc"] = torch.full((self.nlay, self.ncol), -1.0, dtype=torch.float64, device="cuda")
        return o

    def mcica(self, ctx):
        ctx.mcica_subcol_lw_device(self.ncol, self.nlay, self.d, icld=3, permuteseed=self.seed0,
                                   seed_per_column=True)

    def desc(self, mode, out=None):
        arrays = dict(self.d)
        arrays.update(out if out is not None else self.out)
        if mode == R.CLOUD_FUSED:
            arrays["reicmcl"], arrays["relqmcl"] = self.d["rei"], self.d["rel"]
        return R.grid_desc(self.ncol, self.nlay, arrays, icld=3, cloud_mode=mode, seed0=self.seed0)

    def single(self, ctx, out):
        p = dict(self.d)
        p.update(out)
        ctx.rrtmg_lw_device(self.ncol, self.nlay, p)


def _np(out):
    return {k: v.cpu().numpy().T.copy() for k, v in out.items()}


def _same(a, b):
    for k in OUTS:
        assert np.array_equal(a[k], b[k]), (k, float(np.abs(a[k] - b[k]).max()))


@pytest.fixture(scope="module")
def grids(ctx):
    import torch

    gs = [Grid(n, l, s, seed0=1000 * (i + 1)) for i, (n, l, s) in enumerate(GRIDS)]
    for g in gs:
        g.mcica(ctx)
    torch.cuda.synchronize()
    return gs


@pytest.fixture(scope="module")
def singles(ctx, grids):
    import torch

    res = []
    for g in grids:
        o = g.new_out()
        g.single(ctx, o)
        res.append(o)
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    return [_np(o) for o in res]


def test_batch_equals_single_calls(ctx, grids, singles):
    import torch

    ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_SUBCOL) for g in grids])
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    for g, ref in zip(grids, singles):
        _same(_np(g.out), ref)


def test_fused_clouds_equal_mcica_then_rrtmg(ctx, grids, singles):
    import torch

    outs = [g.new_out() for g in grids]
    ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs)])
    torch.cuda.synchronize()
    assert ctx.sync_status() == 0
    for o, ref in zip(outs, singles):
        _same(_np(o), ref)


def test_every_variant_and_grid_size_identical(ctx, grids, singles):
    import torch

    nlay = max(g.nlay for g in grids)
    saved = ctx.tuning(nlay, R.KIND_FUSED)
    try:
        for v in range(ctx.num_variants()):
            for per in (1, 2):
                ctx.set_tuning(nlay, v, per, kind=R.KIND_FUSED)
                outs = [g.new_out() for g in grids]
                ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs)])
                torch.cuda.synchronize()
                for o, ref in zip(outs, singles):
                    _same(_np(o), ref)
    finally:
        ctx.set_tuning(nlay, saved["variant"], saved["blocks_per_sm"], kind=R.KIND_FUSED)
    assert ctx.sync_status() == 0


def test_graph_replay_tracks_inputs_in_place(ctx, grids):
    import torch

    outs_g = [g.new_out() for g in grids]
    graph = ctx.batch_graph([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs_g)])
    try:
        graph.launch()
        outs_d = [g.new_out() for g in grids]
        ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs_d)])
        torch.cuda.synchronize()
        for a, b in zip(outs_g, outs_d):
            _same(_np(a), _np(b))
        before = _np(outs_g[0])["uflx"]
        # a model step: the state changes in place, the graph is replayed
        saved = [(g.d["tlay"].clone(), g.d["tlev"].clone()) for g in grids]
        for g in grids:
            g.d["tlay"].add_(1.5)
            g.d["tlev"].add_(1.5)
        graph.launch()
        ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs_d)])
        torch.cuda.synchronize()
        for a, b in zip(outs_g, outs_d):
            _same(_np(a), _np(b))
        # a warmer atmosphere sends more longwave out at the top
        assert (_np(outs_g[0])["uflx"][:, -1] - before[:, -1]).min() > 0.1
        for g, (tl, tv) in zip(grids, saved):
            g.d["tlay"].copy_(tl)
            g.d["tlev"].copy_(tv)
    finally:
        graph.close()
    assert ctx.sync_status() == 0


def test_autotune_picks_a_valid_shape(ctx, grids, singles):
    import torch

    descs = [g.desc(R.CLOUD_FUSED) for g in grids]
    best = ctx.autotune(descs, sample_cols=0, reps=1)
    assert 0 <= best["variant"] < ctx.num_variants()
    assert best["blocks_per_sm"] >= 1 and best["ms"] > 0
    assert ctx.tuning(max(g.nlay for g in grids), R.KIND_FUSED)["variant"] == best["variant"]
    outs = [g.new_out() for g in grids]
    ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs)])
    torch.cuda.synchronize()
    for o, ref in zip(outs, singles):
        _same(_np(o), ref)
    assert ctx.sync_status() == 0


def test_fused_batch_against_oracle(ctx, grids):
    import torch

    outs = [g.new_out() for g in grids]
    ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED, o) for g, o in zip(grids, outs)])
    torch.cuda.synchronize()
    for g, o in zip(grids, outs):
        mc = pyoracle.mcica_per_column(g.st, g.tauc, icld=3, base_seed=g.seed0)
        ref = pyoracle.rrtmg_lw(g.st, mc, icld=3)
        got = _np(o)
        for k in ("uflx", "dflx", "uflxc", "dflxc"):
            assert np.abs(got[k] - ref[k]).max() <= FLUX_TOL, k
        for k in ("hr", "hrc"):
            assert np.abs(got[k] - ref[k]).max() <= HR_TOL, k


def test_batch_argument_errors(ctx, grids):
    g = grids[0]
    bad = g.desc(R.CLOUD_FUSED)
    bad.icld = 2  # fused clouds are generated with maximum overlap only
    with pytest.raises(R.RrtmgLwError):
        ctx.rrtmg_lw_batch_device([bad])
    with pytest.raises(ValueError):
        ctx.rrtmg_lw_batch_device([])
    with pytest.raises(ValueError):
        ctx.rrtmg_lw_batch_device([g.desc(R.CLOUD_FUSED)] * (R.MAX_GRIDS + 1))
    with pytest.raises(R.RrtmgLwError):
        ctx.set_tuning(g.nlay, ctx.num_variants(), 1)
    with pytest.raises(R.RrtmgLwError):
        ctx.set_tuning(g.nlay, 0, 1, kind=4)
