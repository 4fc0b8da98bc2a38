"""Column sharding across GPUs (one process per GPU, no data-path collective).

Columns are independent (each MPI rank of BRAMS already solves its own
subdomain, rtm_driver.f90:830), so a multi-GPU run gives every rank a
contiguous range of columns.  Ranges are balanced by work, which is
proportional to the number of layers of each column when grids of
different depth are batched together.
"""
from __future__ import annotations

import numpy as np


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
