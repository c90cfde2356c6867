"""The GPU planner (idg_plan_subgrids) against the host planner
(datasets.plan_subgrids_split): every plan entry and channel range identical,
bit for bit, on the config-3 generator (100 km baselines, 64 channels over
100-200 MHz, S = 32 and 64) -- shrunk to 12 stations, and as the sample of the
full 100-station geometry that reaches 97.6 km -- and on config-2 geometry
(10 km, 16 channels, A-term slots every 256 steps)."""
import dataclasses

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _cases():
    from idg_gb300 import datasets as D

    return [
        ("config3 S=32", D.config3(32, nstations=12, ntimesteps=512)),
        ("config3 S=64", D.config3(64, nstations=12, ntimesteps=512)),
        ("config2 30 stations", dataclasses.replace(D.config2(), nstations=30, ntimesteps=2048)),
    ]


@pytest.mark.parametrize("case", range(3))
def test_gpu_plan_matches_host_plan(idg, case):
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    name, spec = _cases()[case]
    obs = D.make_observation(spec)  # geometry (the fixed-length plan is not used)
    want_md, want_ext = D.plan_subgrids_split(spec, obs.uvw, obs.frequencies, obs.baselines)
    md, ext = ops.plan_subgrids(torch.from_numpy(obs.uvw).cuda(), torch.from_numpy(obs.frequencies).cuda(),
                                torch.from_numpy(obs.baselines.astype(np.int32)).cuda(), spec.ntimesteps,
                                spec.subgrid_size, spec.grid_size, spec.image_size, spec.timesteps_per_subgrid,
                                spec.aterm_interval)
    print(f"[planner] {name}: {md.shape[0]} subgrids on the GPU, {want_md.shape[0]} on the host")
    assert md.shape == want_md.shape
    for f in want_md.dtype.names:
        assert np.array_equal(md[f], want_md[f]), f
    assert np.array_equal(ext, want_ext)


@pytest.mark.parametrize("S", [32, 64])
def test_gpu_plan_matches_host_plan_at_100_km(idg, S):
    """The longest baselines of the full config-3 geometry: at 200 MHz their
    tracks cross a subgrid in under a minute and a channel group holds one to
    four channels (S = 32)."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    obs, _, _, lengths = D.config3_sample(S)
    spec = obs.spec
    assert lengths.max() >= 95e3
    md, ext = ops.plan_subgrids(torch.from_numpy(obs.uvw).cuda(), torch.from_numpy(obs.frequencies).cuda(),
                                torch.from_numpy(obs.baselines.astype(np.int32)).cuda(), spec.ntimesteps, S,
                                spec.grid_size, spec.image_size, spec.timesteps_per_subgrid, spec.aterm_interval)
    print(f"[planner] config3 sample to {lengths.max() / 1e3:.1f} km, S={S}: {md.shape[0]} subgrids")
    assert md.shape == obs.metadata.shape
    for f in obs.metadata.dtype.names:
        assert np.array_equal(md[f], obs.metadata[f]), f
    assert np.array_equal(ext, obs.ext)


def test_gpu_plan_reports_the_needed_capacity(idg):
    import idg_gb300._lib as L
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config3(32, nstations=6, ntimesteps=256)
    obs = D.make_observation(spec)
    args = (torch.from_numpy(obs.uvw).cuda(), torch.from_numpy(obs.frequencies).cuda(),
            torch.from_numpy(obs.baselines.astype(np.int32)).cuda(), spec.ntimesteps, spec.subgrid_size,
            spec.grid_size, spec.image_size, spec.timesteps_per_subgrid, spec.aterm_interval)
    md, _ = ops.plan_subgrids(*args)
    with pytest.raises(L.IdgError) as e:
        ops.plan_subgrids(*args, capacity=md.shape[0] - 1)
    assert e.value.code == L.IDG_ERR_INVALID_ARGUMENT and "max_subgrids" in str(e.value)


def test_gpu_plan_full_config2(idg):
    """The full config-2 geometry (4950 baselines x 8192 steps) planned on the GPU:
    every visibility in some subgrid (sample count), entries in (baseline, time)
    order, A-term slots respected, and the planning time printed."""
    import time

    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config2()
    obs = D.make_observation(spec)
    args = (torch.from_numpy(obs.uvw).cuda(), torch.from_numpy(obs.frequencies).cuda(),
            torch.from_numpy(obs.baselines.astype(np.int32)).cuda(), spec.ntimesteps, spec.subgrid_size,
            spec.grid_size, spec.image_size, spec.timesteps_per_subgrid, spec.aterm_interval)
    ops.plan_subgrids(*args)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    md, ext = ops.plan_subgrids(*args)
    ms = (time.perf_counter() - t0) * 1e3
    print(f"[planner] config2 full: {md.shape[0]} subgrids in {ms:.1f} ms (GPU planner incl. count, scan, copy-back)")
    nvis = int(((ext["channel_end"] - ext["channel_begin"]).astype(np.int64) * md["nr_timesteps"]).sum())
    assert nvis == spec.n_baselines * spec.ntimesteps * spec.nchannels
    assert np.all(np.diff(md["time_offset"].astype(np.int64) // spec.ntimesteps) >= 0)  # baseline order
    t_in = md["time_offset"] % spec.ntimesteps
    assert np.all(t_in // spec.aterm_interval == (t_in + md["nr_timesteps"] - 1) // spec.aterm_interval)
    S, G = spec.subgrid_size, spec.grid_size
    assert (md["x"] >= 0).all() and (md["x"] + S <= G).all()
