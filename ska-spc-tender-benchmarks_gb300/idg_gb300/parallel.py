"""Sharding the IDG path over several GPUs (one process per GPU).

Subgrids are independent for the gridder, the degridder and the subgrid FFT;
only the adder has an exchange step (every rank adds its subgrids into its own
copy of the uv-grid, then the copies are summed).  The plan is partitioned by
grid-tile ownership so that most of a rank's subgrids land on its own tiles:

* ``partition_plan`` assigns each subgrid to the owner of the grid tile that
  holds the subgrid's centre; tiles are dealt to ranks greedily, heaviest
  first, by their visibility count (longest-processing-time order), so the
  ranks carry near-equal work.
* ``reduce_grid`` sums the per-rank grids with one all-reduce
  (``torch.distributed``: NCCL between GPUs, gloo on CPU); degridding then
  needs the full grid on every rank, which the all-reduce provides.
"""
from __future__ import annotations

import numpy as np

from ._lib import METADATA_DTYPE


def subgrid_work(metadata: np.ndarray, nr_channels: int, ext: np.ndarray | None = None) -> np.ndarray:
    """Visibilities per subgrid (the gridder's cost is proportional to this times S^2)."""
    md = np.asarray(metadata, METADATA_DTYPE)
    nch = np.full(md.shape[0], nr_channels, np.int64) if ext is None else (ext["channel_end"] - ext["channel_begin"]).astype(np.int64)
    return md["nr_timesteps"].astype(np.int64) * nch


def partition_plan(metadata: np.ndarray, world_size: int, subgrid_size: int, tile: int = 64,
                   nr_channels: int = 1, ext: np.ndarray | None = None) -> list[np.ndarray]:
    """Subgrid indices per rank (each sorted ascending), balanced by visibility count."""
    md = np.asarray(metadata, METADATA_DTYPE)
    n = md.shape[0]
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    if n == 0:
        return [np.zeros(0, np.int64) for _ in range(world_size)]
    cx = (md["x"].astype(np.int64) + subgrid_size // 2) // tile
    cy = (md["y"].astype(np.int64) + subgrid_size // 2) // tile
    key = (cy - cy.min()) * (int(cx.max() - cx.min()) + 1) + (cx - cx.min())
    tiles, inverse = np.unique(key, return_inverse=True)
    work = subgrid_work(md, nr_channels, ext)
    tile_work = np.bincount(inverse, weights=work, minlength=len(tiles))
    owner = np.empty(len(tiles), np.int64)
    load = np.zeros(world_size)
    for t in np.argsort(-tile_work, kind="stable"):
        r = int(np.argmin(load))
        owner[t] = r
        load[r] += tile_work[t]
    rank_of = owner[inverse]
    return [np.nonzero(rank_of == r)[0] for r in range(world_size)]


def reduce_grid(grid, group=None):
    """Sum a [W,4,G,G] complex64 grid tensor over all ranks, in place (all-reduce)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return grid
    view = torch.view_as_real(grid) if grid.is_complex() else grid
    dist.all_reduce(view, op=dist.ReduceOp.SUM, group=group)
    return grid
