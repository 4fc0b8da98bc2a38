"""Multi-GPU column shards through the library on one GPU.

Each rank of a multi-GPU caller solves the slices that gb_rrtmg_lw_shard_plan
gives it (gb_rrtmg_lw_grid_slice descriptors) with one batched launch on its
own device.  Columns are independent and the McICA seeds advance with the
slice, so the union of the ranks' outputs must equal one unsharded batched
call bit for bit.  One GPU runs the ranks' launches one after another (no
launch waits on another).
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu

SHAPES = [(300, 45), (170, 38), (91, 60)]
OUTS = ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "hr", "hrc")


def _grids(seed):
    from brams_gb300 import surrogate as S

    out = []
    for i, (nc, nl) in enumerate(SHAPES):
        st = make_state(ProfileSpec(ncol=nc, nlay=nl, seed=seed + i, t_noise=4.0, h2o_sigma=0.5, cloud_prob=0.6))
        st["tauaer"] = np.asfortranarray(np.random.default_rng(seed + i).uniform(0.0, 0.02, st["tauaer"].shape))
        out.append(S.DeviceGrid(st, pyoracle.cldprop_columns(st)))
    return out


@pytest.mark.parametrize("world", [2, 3, 5])
def test_sharded_batch_equals_unsharded(ctx, world):
    import torch

    from brams_gb300.shard import solve_shard

    whole, parts = _grids(60), _grids(60)
    ctx.rrtmg_lw_batch_device([g.desc(seed0=100 * (i + 1)) for i, g in enumerate(whole)])
    descs = [g.desc(seed0=100 * (i + 1)) for i, g in enumerate(parts)]
    solved = [0] * len(SHAPES)
    for rank in range(world):
        for gi, d in solve_shard(ctx, descs, world=world, rank=rank):
            solved[gi] += d.ncol
    torch.cuda.synchronize()
    assert solved == [nc for nc, _ in SHAPES]
    for a, b in zip(whole, parts):
        for k in OUTS:
            assert torch.equal(a.d[k], b.d[k]), k
    assert ctx.sync_status() == 0


def test_sharded_learned_batch_equals_unsharded(ctx):
    """Learned gas optics (gb_rrtmg_lw_batch_surrogate) on the slices."""
    import torch

    from brams_gb300 import surrogate as S
    from brams_gb300.shard import solve_shard

    mlp = S.load(ctx)
    whole, parts = _grids(70), _grids(70)
    mlp.batch([g.desc(seed0=7 + i) for i, g in enumerate(whole)])
    descs = [g.desc(seed0=7 + i) for i, g in enumerate(parts)]
    for rank in range(2):
        solve_shard(ctx, descs, world=2, rank=rank, mlp=mlp)
    torch.cuda.synchronize()
    for a, b in zip(whole, parts):
        for k in OUTS:
            assert torch.equal(a.d[k], b.d[k]), k
    mlp.close()
