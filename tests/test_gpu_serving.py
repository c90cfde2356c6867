"""Serving: jobs admitted while others run -- their kernels overlapping on the
GPU, shown by the jobs' device intervals -- give the same results as the same
jobs run alone, bit for bit (the jobs' adders sum in a fixed order, and the
other kernels give each output a fixed summation order whatever share of the
SMs they get), a grid can be read while jobs on it are still running, jobs
larger than the HBM budget are rejected, and latency statistics are kept."""
import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from conftest import check_rel

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _job(seed, nstations, ntimesteps, nchannels, grid_size=1024):
    from idg_gb300 import datasets as D
    from idg_gb300.ops import GridSpec
    from idg_gb300.serving import JobData

    spec = D.ObservationSpec(nstations=nstations, disk_radius_m=2000.0, ntimesteps=ntimesteps,
                             timesteps_per_subgrid=32, nchannels=nchannels, f_start=150e6, f_end=160e6,
                             subgrid_size=32, grid_size=grid_size, image_size=0.05, aterm_sigma=0.05,
                             aterm_interval=64, seed=seed)
    obs = D.make_observation(spec)
    rng = np.random.default_rng(seed)
    vis = (rng.standard_normal((spec.n_rows, nchannels, 4)) + 1j * rng.standard_normal((spec.n_rows, nchannels, 4))).astype(np.complex64)
    gs = GridSpec(grid_size, 32, nchannels, nstations, obs.aterms.shape[0], 1, spec.image_size)
    grid_in = JobData(gs, obs.metadata, obs.uvw, obs.wavenumbers, obs.taper, np.ascontiguousarray(obs.aterms), vis)
    out = np.zeros_like(vis)
    degrid = JobData(gs, obs.metadata, obs.uvw, obs.wavenumbers, obs.taper, np.ascontiguousarray(obs.aterms), out)
    return grid_in, degrid


# (seed, stations, timesteps, channels): 600-1150 subgrids of 32 timesteps each,
# large enough that a job's kernels run for a good part of a millisecond
JOBS = [(1, 16, 256, 16), (2, 20, 192, 8), (3, 12, 512, 24), (4, 18, 128, 16)]


def _run(server, jobs, together):
    """Grid every job into its own resident grid, then degrid from it.
    Returns the grids and visibilities, and each job's statistics."""
    grids = [server.grid_create(1024) for _ in jobs]
    stats = []
    if together:
        ids = [server.submit(L.IDG_JOB_GRID, g, gid) for (g, _), gid in zip(jobs, grids)]
        ids += [server.submit(L.IDG_JOB_DEGRID, d, gid) for (_, d), gid in zip(jobs, grids)]
        stats = [server.wait(i, 120) for i in ids]
    else:
        for (g, d), gid in zip(jobs, grids):
            stats.append(server.wait(server.submit(L.IDG_JOB_GRID, g, gid), 120))
            stats.append(server.wait(server.submit(L.IDG_JOB_DEGRID, d, gid), 120))
    out = [(server.grid_read(gid, 1024), d.vis.copy()) for (_, d), gid in zip(jobs, grids)]
    for gid in grids:
        server.grid_release(gid)
    return out, stats


def _overlapping_pairs(stats):
    """Pairs of jobs whose kernels' device intervals intersect."""
    iv = [(s["device_start_ms"], s["device_end_ms"]) for s in stats]
    assert all(0 <= a < b for a, b in iv), iv
    return [(i, j) for i in range(len(iv)) for j in range(i + 1, len(iv))
            if max(iv[i][0], iv[j][0]) < min(iv[i][1], iv[j][1])]


def test_jobs_alone_and_in_the_mix_agree(idg):
    from idg_gb300.serving import Server

    jobs = [_job(*j) for j in JOBS]
    with Server(max_slots=1, hbm_budget_bytes=8 << 30) as s1:
        alone, job_alone = _run(s1, jobs, together=False)
        st1 = s1.stats()
    # one slot: every job runs alone on the GPU
    assert _overlapping_pairs(job_alone) == []
    for _, d in jobs:
        d.vis[...] = 0
    with Server(max_slots=4, hbm_budget_bytes=8 << 30, cta_share=True) as s4:
        mixed, job_mixed = _run(s4, jobs, together=True)
        st4 = s4.stats()
    pairs = _overlapping_pairs(job_mixed)
    print(f"[serving] jobs whose kernels overlapped on the GPU: {pairs}")
    assert pairs, "no two jobs' kernels ran at the same time"
    for k, ((ga, va), (gm, vm)) in enumerate(zip(alone, mixed)):
        assert np.abs(ga).max() > 0 and np.abs(va).max() > 0
        check_rel(f"serving job {k} grid alone vs mix", gm, ga, TOL)
        check_rel(f"serving job {k} vis alone vs mix", vm, va, TOL)
        assert np.array_equal(gm, ga), f"job {k}: grid alone and in the mix differ"
        assert np.array_equal(vm, va), f"job {k}: visibilities alone and in the mix differ"
    assert st1["completed"] == st4["completed"] == 2 * len(JOBS)
    assert st4["p99_ms"] >= st4["p50_ms"] > 0
    assert st4["hbm_peak"] > 0


def test_serving_result_matches_direct_plan(idg):
    """A served gridding + degridding job equals the plan API on the same data."""
    from idg_gb300 import ops
    from idg_gb300.serving import Server

    g, d = _job(7, 6, 128, 16)
    with Server(max_slots=2, hbm_budget_bytes=4 << 30) as s:
        gid = s.grid_create(1024)
        s.wait(s.submit(L.IDG_JOB_GRID, g, gid), 120)
        s.wait(s.submit(L.IDG_JOB_DEGRID, d, gid), 120)
        grid_srv = s.grid_read(gid, 1024)
    dv = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
          dict(uvw=g.uvw, k=g.wavenumbers, vis=g.vis, taper=g.taper, at=g.aterms).items()}
    plan = ops.Plan(g.spec, g.metadata, g.nr_rows)
    grid = torch.zeros((1, 4, 1024, 1024), dtype=torch.complex64, device="cuda")
    plan.grid(dv["uvw"], dv["k"], dv["vis"], dv["taper"], dv["at"], grid)
    vout = torch.zeros_like(dv["vis"])
    plan.degrid(dv["uvw"], dv["k"], vout, dv["taper"], dv["at"], grid)
    torch.cuda.synchronize()
    check_rel("served grid vs plan", grid_srv, grid.cpu().numpy(), TOL)
    check_rel("served vis vs plan", d.vis, vout.cpu().numpy(), TOL)
    plan.close()


def test_grid_read_while_jobs_run(idg):
    """grid_read called right after submission, while the gridding job runs,
    waits for it and returns its complete grid; a read beside a running
    degridding job (which does not change the grid) returns the same bytes."""
    from idg_gb300.serving import Server

    g, d = _job(11, 24, 512, 16)
    with Server(max_slots=2, hbm_budget_bytes=8 << 30) as s:
        gid = s.grid_create(1024)
        jg = s.submit(L.IDG_JOB_GRID, g, gid)
        early = s.grid_read(gid, 1024)
        s.wait(jg, 120)
        after = s.grid_read(gid, 1024)
        jd = s.submit(L.IDG_JOB_DEGRID, d, gid)
        beside = s.grid_read(gid, 1024)
        s.wait(jd, 120)
        s.grid_release(gid)
    assert np.abs(after).max() > 0
    assert np.array_equal(early, after)
    assert np.array_equal(beside, after)


def test_job_over_budget_is_rejected(idg):
    from idg_gb300.serving import Server

    g, _ = _job(5, 8, 256, 16)  # ~11 MB of device memory
    with Server(max_slots=2, hbm_budget_bytes=4 << 20) as s:
        gid = s.grid_create(1024)
        with pytest.raises(L.IdgError) as e:
            s.submit(L.IDG_JOB_GRID, g, gid)
        assert e.value.code == L.IDG_ERR_REJECTED
        assert s.stats()["rejected"] == 1
