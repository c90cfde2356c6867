"""The sharded imaging cycle on the product kernels: two gloo ranks, each a
process on the one GPU of this machine, run parallel.sharded_cycle -- the
tile-owner partition of the plan, the CUDA gridding step of its own subgrids,
the grid all-reduce, the CUDA degridding step of its own subgrids -- and the
summed grid and the ranks' visibilities together equal one process running
the whole plan through the same kernels (within 1e-6: the adder's
floating-point atomics may sum in another order).  The ranks' kernels never
wait on one another; the all-reduce runs on the host."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT, check_rel

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _problem():
    from idg_gb300 import datasets as D

    spec = D.ObservationSpec(nstations=12, disk_radius_m=1500.0, ntimesteps=256, timesteps_per_subgrid=32,
                             nchannels=8, f_start=150e6, f_end=160e6, subgrid_size=32, grid_size=1024,
                             image_size=0.05, aterm_sigma=0.05, aterm_interval=128, seed=31)
    obs = D.make_observation(spec)
    rng = np.random.default_rng(32)
    vis = (rng.standard_normal((spec.n_rows, spec.nchannels, 4)) +
           1j * rng.standard_normal((spec.n_rows, spec.nchannels, 4))).astype(np.complex64)
    return spec, obs, vis


def _device_inputs(spec, obs, vis):
    import torch

    from idg_gb300 import ops

    gs = ops.GridSpec(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, obs.aterms.shape[0], 1,
                      spec.image_size)
    d = dict(uvw=torch.from_numpy(obs.uvw).cuda(), k=torch.from_numpy(obs.wavenumbers).cuda(),
             vis=torch.from_numpy(vis).cuda(), taper=torch.from_numpy(obs.taper).cuda(),
             at=torch.from_numpy(np.ascontiguousarray(obs.aterms)).cuda())
    return gs, d


def _rank_main(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, os.path.join(ROOT, "ska-spc-tender-benchmarks_gb300"))
    import torch
    import torch.distributed as dist

    from idg_gb300 import parallel

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    spec, obs, vis = _problem()
    gs, d = _device_inputs(spec, obs, vis)
    grid = torch.empty((1, 4, spec.grid_size, spec.grid_size), dtype=torch.complex64, device="cuda")
    vout = torch.zeros_like(d["vis"])
    mine = parallel.sharded_cycle(gs, obs.metadata, d["uvw"], d["k"], d["vis"], d["taper"], d["at"], grid, vout)
    torch.cuda.synchronize()
    np.save(os.path.join(out_dir, f"grid_{rank}.npy"), grid.cpu().numpy())
    np.save(os.path.join(out_dir, f"vis_{rank}.npy"), vout.cpu().numpy())
    np.save(os.path.join(out_dir, f"mine_{rank}.npy"), mine)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_on_the_product_kernels_equal_one(idg, tmp_path):
    import torch

    from idg_gb300 import ops

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    spec, obs, vis = _problem()
    mine = [np.load(tmp_path / f"mine_{r}.npy") for r in range(2)]
    assert len(mine[0]) > 0 and len(mine[1]) > 0
    assert np.array_equal(np.sort(np.concatenate(mine)), np.arange(spec.n_subgrids))
    g0, g1 = np.load(tmp_path / "grid_0.npy"), np.load(tmp_path / "grid_1.npy")
    assert np.array_equal(g0, g1)  # every rank holds the same summed grid

    # one process, the whole plan, the same kernels
    gs, d = _device_inputs(spec, obs, vis)
    md = ops.metadata_tensor(obs.metadata, "cuda")
    S = spec.subgrid_size
    sub = torch.empty((spec.n_subgrids, 4, S, S), dtype=torch.complex64, device="cuda")
    grid = torch.zeros((1, 4, spec.grid_size, spec.grid_size), dtype=torch.complex64, device="cuda")
    ops.grid_visibilities(gs, md, d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, grid)
    vout = torch.zeros_like(d["vis"])
    ops.degrid_visibilities(gs, md, d["uvw"], d["k"], vout, d["taper"], d["at"], sub, grid)
    torch.cuda.synchronize()
    check_rel("sharded grid (2 ranks) vs one process", g0, grid.cpu().numpy(), 1e-6)
    # each rank wrote the rows of its own subgrids; together they are the whole output
    v = [np.load(tmp_path / f"vis_{r}.npy") for r in range(2)]
    rows = np.zeros(spec.n_rows, np.int64)
    for r in range(2):
        for m in obs.metadata[mine[r]]:
            rows[m["time_offset"]:m["time_offset"] + m["nr_timesteps"]] = r
    combined = np.where(rows[:, None, None] == 0, v[0], v[1])
    check_rel("sharded visibilities (2 ranks) vs one process", combined, vout.cpu().numpy(), 1e-6)
