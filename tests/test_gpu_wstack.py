"""w-stacking end to end against the FP64 oracle.

A split plan with w-planes (z = floor(w_mid / w_step) clipped to [-W, W-1];
negative z go to the Hermitian-mirrored plane -z-1) is gridded through
idg_grid_visibilities (gridder -> subgrid FFT +1 -> adder) into a
[W][4][G][G] grid, and a random grid is predicted back through
idg_degrid_visibilities (splitter -> subgrid FFT -1 -> degridder).  The
oracle runs the same steps in FP64: gridder / degridder with the w offset
(z + 1/2) w_step, the direct subgrid DFT, and the adder / splitter with the
mirror rule.  Both variants; relative RMS <= 1e-5 for grid and visibilities.
The GPU planner gives the same w-plane indices as the host planner.
"""
import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from conftest import check_rel
from gpu_helpers import dev, spec_for
from test_gpu_kernels import _oracle_with_ext

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _wstack_obs():
    from idg_gb300 import datasets as D

    spec = D.ObservationSpec(nstations=8, disk_radius_m=2500.0, ntimesteps=256, timesteps_per_subgrid=64,
                             nchannels=16, f_start=140e6, f_end=170e6, subgrid_size=32, grid_size=512,
                             image_size=0.04, w_step=300.0, nr_w_planes=4, aterm_sigma=0.05, aterm_interval=128,
                             dec_deg=20.0, seed=5)
    return spec, D.make_observation(spec, split=True)


def test_wstacked_grid_and_degrid_vs_oracle(oracle_mod, idg):
    from idg_gb300 import ops

    spec, obs = _wstack_obs()
    md, ext = obs.metadata, obs.ext
    G, S, C, W = spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nr_w_planes
    w_step = float(np.float32(spec.w_step))
    assert (md["z"] < 0).any() and (md["z"] >= 0).any()
    assert md["z"].min() >= -W and md["z"].max() <= W - 1
    print(f"[w-stack] {md.shape[0]} subgrids, z histogram {np.bincount(md['z'] + W, minlength=2 * W).tolist()}")
    rows = obs.uvw.shape[0]
    rng = np.random.default_rng(9)
    vis = (rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64)
    g_in = (rng.standard_normal((W, 4, G, G)) + 1j * rng.standard_normal((W, 4, G, G))).astype(np.complex64)

    # oracle: gridder (taper) -> DFT +1 -> adder; splitter -> DFT -1 -> degridder (taper)
    sub_in = oracle_mod.subgrid_dft(oracle_mod.splitter(g_in, md, S), -1).astype(np.complex64)
    want_sub, want_vis = _oracle_with_ext(oracle_mod, G, S, spec.nstations, spec.image_size, obs.uvw,
                                          obs.wavenumbers, vis, obs.taper, obs.aterms, md, ext, sub_in, w_step)
    want_grid = oracle_mod.adder(oracle_mod.subgrid_dft(want_sub, +1), md, G, W)

    sp = spec_for(G, S, C, spec.nstations, obs.aterms.shape[0], spec.image_size, w_step=w_step, W=W)
    N = md.shape[0]
    args = (dev(md), dev(obs.uvw), dev(obs.wavenumbers))
    for variant in (L.VARIANT_PLAIN, L.VARIANT_BATCHED):
        grid = torch.zeros((W, 4, G, G), dtype=torch.complex64, device="cuda")
        sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
        ops.grid_visibilities(sp, *args, dev(vis), dev(obs.taper), dev(obs.aterms), sub, grid, variant=variant,
                              ext=ops.ext_tensor(ext, "cuda"))
        v_out = torch.zeros((rows, C, 4), dtype=torch.complex64, device="cuda")
        ops.degrid_visibilities(sp, *args, v_out, dev(obs.taper), dev(obs.aterms), sub, dev(g_in), variant=variant,
                                ext=ops.ext_tensor(ext, "cuda"))
        torch.cuda.synchronize()
        check_rel(f"w-stacked grid v{variant}", grid.cpu().numpy(), want_grid, TOL)
        check_rel(f"w-stacked degrid v{variant}", v_out.cpu().numpy(), want_vis, TOL)
        # every plane receives data; the mirrored entries land in planes too
        assert all(np.abs(grid[p].cpu().numpy()).max() > 0 for p in np.unique(np.where(md["z"] < 0, -md["z"] - 1,
                                                                                      md["z"])))


def test_gpu_planner_w_planes_match_host(idg):
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec, obs = _wstack_obs()
    want_md, want_ext = D.plan_subgrids_split(spec, obs.uvw, obs.frequencies, obs.baselines)
    md, ext = ops.plan_subgrids(torch.from_numpy(obs.uvw).cuda(), torch.from_numpy(obs.frequencies).cuda(),
                                torch.from_numpy(obs.baselines.astype(np.int32)).cuda(), spec.ntimesteps,
                                spec.subgrid_size, spec.grid_size, spec.image_size, spec.timesteps_per_subgrid,
                                spec.aterm_interval, w_step=spec.w_step, nr_w_planes=spec.nr_w_planes)
    assert (want_md["z"] < 0).any()
    for f in want_md.dtype.names:
        assert np.array_equal(md[f], want_md[f]), f
    assert np.array_equal(ext, want_ext)


def test_wstacked_plan_graph_cycle_matches_direct_steps(idg):
    """A device-resident plan with w-planes (negative z mirrored) replays its
    grid + degrid cycle as one CUDA graph with the same grid and predicted
    visibilities as the direct steps (gridding, then degridding from that grid)."""
    from idg_gb300 import ops

    spec, obs = _wstack_obs()
    md, ext = obs.metadata, obs.ext
    G, S, C, W = spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nr_w_planes
    sp = spec_for(G, S, C, spec.nstations, obs.aterms.shape[0], spec.image_size, w_step=float(np.float32(spec.w_step)),
                  W=W)
    rows, N = obs.uvw.shape[0], md.shape[0]
    rng = np.random.default_rng(10)
    vis = dev((rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64))
    d = dict(md=dev(md), uvw=dev(obs.uvw), k=dev(obs.wavenumbers), taper=dev(obs.taper), at=dev(obs.aterms),
             ext=ops.ext_tensor(ext, "cuda"))
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    g_ref = torch.zeros((W, 4, G, G), dtype=torch.complex64, device="cuda")
    ops.grid_visibilities(sp, d["md"], d["uvw"], d["k"], vis, d["taper"], d["at"], sub, g_ref, ext=d["ext"])
    v_ref = torch.zeros_like(vis)
    ops.degrid_visibilities(sp, d["md"], d["uvw"], d["k"], v_ref, d["taper"], d["at"], sub, g_ref, ext=d["ext"])
    plan = ops.Plan(sp, md, rows, ext=ext, variant=L.VARIANT_BATCHED)
    g = torch.full_like(g_ref, 3.0)
    v = torch.zeros_like(vis)
    plan.capture_cycle(d["uvw"], d["k"], vis, d["taper"], d["at"], g, v)
    for _ in range(2):
        plan.launch_cycle()
    torch.cuda.synchronize()
    check_rel("w-stacked graph cycle grid", g.cpu().numpy(), g_ref.cpu().numpy(), TOL)
    check_rel("w-stacked graph cycle vis", v.cpu().numpy(), v_ref.cpu().numpy(), TOL)
    assert plan.status() == 0
    plan.close()
