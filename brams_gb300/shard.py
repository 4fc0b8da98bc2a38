"""Column sharding across GPUs (one process per GPU, no data-path collective).

Columns are independent (each MPI rank of BRAMS already solves its own
subdomain, rtm_driver.f90:830), so a multi-GPU run gives every rank a
contiguous range of columns.  Ranges are balanced by work, which is
proportional to the number of layers of each column when grids of
different depth are batched together.

The plan and the descriptor slices come from the library
(gb_rrtmg_lw_shard_plan, gb_rrtmg_lw_grid_slice), so that a Fortran or C
caller gets the same split; `solve_shard` is what one rank runs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import rrtmg_lw as R


def balanced_ranges(work: np.ndarray, world: int) -> list[tuple[int, int]]:
    """Split items 0..n-1 (per-item cost `work`) into `world` contiguous ranges
    of nearly equal total cost.  Returns [(start, stop)) per rank."""
    work = np.asarray(work, dtype=np.float64)
    n = work.size
    if world <= 0:
        raise ValueError("world must be positive")
    if n == 0:
        return [(0, 0)] * world
    csum = np.concatenate([[0.0], np.cumsum(work)])
    total = csum[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        k = int(np.searchsorted(csum, target, side="left"))
        k = min(max(k, bounds[-1]), n)
        bounds.append(k)
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def column_ranges(ncol: int, world: int) -> list[tuple[int, int]]:
    """Equal-depth columns: contiguous ranges of ncol // world (+1)."""
    return balanced_ranges(np.ones(ncol), world)


def shard_plan(shapes, world: int, rank: int) -> list[tuple[int, int]]:
    """Per grid (ncol, nlay) of a batch, the column range [c0, c1) that rank
    `rank` of `world` solves (gb_rrtmg_lw_shard_plan)."""
    L = R.load_library()
    n = len(shapes)
    nc = (C.c_int * max(n, 1))(*[int(a) for a, _ in shapes])
    nl = (C.c_int * max(n, 1))(*[int(b) for _, b in shapes])
    c0 = (C.c_int64 * max(n, 1))()
    c1 = (C.c_int64 * max(n, 1))()
    rc = L.gb_rrtmg_lw_shard_plan(n, nc, nl, world, rank, c0, c1)
    if rc != 0:
        raise R.RrtmgLwError(rc, L.gb_rrtmg_lw_strerror(rc).decode())
    return [(c0[i], c1[i]) for i in range(n)]


def slice_grid(g: R.GridDesc, c0: int, c1: int) -> R.GridDesc:
    """Descriptor of columns [c0, c1) of grid g (gb_rrtmg_lw_grid_slice)."""
    L = R.load_library()
    out = R.GridDesc()
    rc = L.gb_rrtmg_lw_grid_slice(C.byref(g), c0, c1, C.byref(out))
    if rc != 0:
        raise R.RrtmgLwError(rc, L.gb_rrtmg_lw_strerror(rc).decode())
    return out


def shard_grids(grids, world: int, rank: int) -> list[tuple[int, R.GridDesc]]:
    """The non-empty slices rank `rank` solves, as (grid index, descriptor)."""
    plan = shard_plan([(g.ncol, g.nlay) for g in grids], world, rank)
    return [(i, slice_grid(g, a, b)) for i, (g, (a, b)) in enumerate(zip(grids, plan)) if b > a]


def solve_shard(ctx: R.Context, grids, world: int | None = None, rank: int | None = None, stream=None,
                mlp: R.Mlp | None = None) -> list[tuple[int, R.GridDesc]]:
    """One rank's part of a batched call: its slices of `grids` in one
    persistent launch on this process's device (rank and world default to
    torch.distributed's).  With `mlp` the slices run on the learned gas
    optics (gb_rrtmg_lw_batch_surrogate).  Returns the slices solved."""
    if world is None or rank is None:
        import torch.distributed as dist

        world, rank = (dist.get_world_size(), dist.get_rank()) if dist.is_initialized() else (1, 0)
    mine = shard_grids(grids, world, rank)
    if mine:
        descs = [d for _, d in mine]
        if mlp is None:
            ctx.rrtmg_lw_batch_device(descs, stream=stream)
        else:
            mlp.batch(descs, stream=stream)
    return mine
