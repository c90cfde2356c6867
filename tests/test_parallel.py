"""The multi-rank path on CPU: plan partition by grid tiles and the grid
all-reduce, run as two gloo ranks; the summed per-rank grids equal the
single-rank grid (FP64 oracle pipeline: gridder -> DFT -> adder)."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _problem():
    from idg_gb300 import datasets as D

    spec = D.config1()
    spec.nstations = 6
    spec.ntimesteps = 32
    spec.timesteps_per_subgrid = 8
    spec.nchannels = 4
    obs = D.make_observation(spec)
    rng = np.random.default_rng(0)
    vis = (rng.standard_normal((spec.n_rows, 4, 4)) + 1j * rng.standard_normal((spec.n_rows, 4, 4))).astype(np.complex64)
    return spec, obs, vis


def _grid_of(O, spec, obs, vis, idx):
    md = obs.metadata[idx]
    prm = O.params(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, len(md), spec.image_size)
    sub = O.gridder(prm, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, md)
    f = O.subgrid_dft(sub, +1)
    return O.adder(f, md, spec.grid_size)


def _rank_main(rank, world, port, out_dir):
    import sys

    for p in (os.path.join(ROOT, "ska-spc-tender-benchmarks_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist

    import oracle as O
    from idg_gb300 import parallel

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    spec, obs, vis = _problem()
    parts = parallel.partition_plan(obs.metadata, world, spec.subgrid_size, tile=64, nr_channels=spec.nchannels)
    g = _grid_of(O, spec, obs, vis, parts[rank]).astype(np.complex64)
    t = torch.from_numpy(g)
    parallel.reduce_grid(t)
    np.save(os.path.join(out_dir, f"grid_{rank}.npy"), t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_partition_covers_plan_and_balances(idg):
    from idg_gb300 import parallel

    spec, obs, _ = _problem()
    for world in (1, 2, 3, 4):
        parts = parallel.partition_plan(obs.metadata, world, spec.subgrid_size, tile=64, nr_channels=4)
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(spec.n_subgrids))
    from idg_gb300 import datasets as D

    big = D.make_observation(D.config2())
    parts = parallel.partition_plan(big.metadata, 4, 32, tile=64, nr_channels=16)
    loads = np.array([len(p) for p in parts], float)
    assert loads.max() / loads.mean() < 1.05


def test_two_gloo_ranks_sum_to_single_rank_grid(oracle_mod, idg, tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    g0 = np.load(tmp_path / "grid_0.npy")
    g1 = np.load(tmp_path / "grid_1.npy")
    assert np.array_equal(g0, g1)
    spec, obs, vis = _problem()
    full = _grid_of(oracle_mod, spec, obs, vis, np.arange(spec.n_subgrids))
    rel = np.linalg.norm(g0 - full) / np.linalg.norm(full)
    assert rel < 1e-6
