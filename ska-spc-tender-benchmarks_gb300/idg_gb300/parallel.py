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
* ``sharded_cycle`` is one imaging cycle on the product kernels: each rank
  grids its part of the plan into its own grid (gridder -> subgrid FFT ->
  adder), the grids are summed, and each rank degrids its part from the sum.
  The all-reduce is the only exchange; no kernel waits on another rank.
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
    """Sum a [W,4,G,G] complex64 grid tensor over all ranks, in place (all-reduce).
    A device grid under a gloo process group goes through host memory, after
    the work queued on the current stream."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return grid
    if grid.is_cuda and dist.get_backend(group) == "gloo":
        torch.cuda.current_stream(grid.device).synchronize()
        host = grid.cpu()
        dist.all_reduce(torch.view_as_real(host), op=dist.ReduceOp.SUM, group=group)
        grid.copy_(host)
        return grid
    view = torch.view_as_real(grid) if grid.is_complex() else grid
    dist.all_reduce(view, op=dist.ReduceOp.SUM, group=group)
    return grid


def _rank_and_world(group=None) -> tuple[int, int]:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def sharded_cycle(spec, metadata: np.ndarray, uvw, wavenumbers, vis, taper, aterms, grid, vis_out,
                  ext: np.ndarray | None = None, tile: int = 64, variant: int | None = None, group=None) -> np.ndarray:
    """One imaging cycle of an observation whose inputs every rank holds (device
    tensors in the layouts of ``ops``), with its subgrids shared out by
    ``partition_plan``: this rank grids its subgrids with the CUDA kernels into
    ``grid`` (zeroed first), the ranks' grids are summed in place
    (``reduce_grid``), and this rank degrids its subgrids from the summed grid
    into ``vis_out`` (the rows and channels its subgrids name; other entries
    are left as they are).  Runs on the current stream.  Returns this rank's
    subgrid indices into ``metadata``."""
    import torch

    from . import _lib, ops

    if variant is None:
        variant = _lib.VARIANT_BATCHED
    rank, world = _rank_and_world(group)
    md = np.asarray(metadata, METADATA_DTYPE)
    mine = partition_plan(md, world, spec.subgrid_size, tile, spec.nr_channels, ext)[rank]
    dev = grid.device
    grid.zero_()
    sub = d_md = d_ext = None
    if len(mine):
        d_md = ops.metadata_tensor(md[mine], dev)
        d_ext = ops.ext_tensor(ext[mine], dev) if ext is not None else None
        sub = torch.empty((len(mine), 4, spec.subgrid_size, spec.subgrid_size), dtype=torch.complex64, device=dev)
        ops.grid_visibilities(spec, d_md, uvw, wavenumbers, vis, taper, aterms, sub, grid, variant=variant, ext=d_ext)
    reduce_grid(grid, group)
    if len(mine):
        ops.degrid_visibilities(spec, d_md, uvw, wavenumbers, vis_out, taper, aterms, sub, grid, variant=variant,
                                ext=d_ext)
    return mine
