"""Serving benchmark: a Poisson stream of gridding and degridding jobs.

    python -m idg_gb300.serve_bench [--rates 2,4,8] [--jobs 24] [--slots 4] [--budget-gb 96]
                                    [--max-vis 1.3e8] [--seed 5]

Each job is an observation drawn from the 100-station generator family:
stations uniform in [16, 200], timesteps uniform in [64, 2048] (whole
64-step subgrids), channels uniform in [8, 64] over 150-160 MHz, and a grid of
1024^2, 2048^2, 4096^2 or 8192^2 cells; the station disk is scaled with the
grid (10 km across at 4096^2) so that every subgrid lands inside it.  A job's
visibility count is capped at --max-vis by shortening its time axis (the cap
keeps host-side data generation to seconds).  Every observation is first
gridded into its own device-resident uv-grid and later degridded from it;
the gridding and degridding jobs of all observations are interleaved in one
stream whose arrival times are exponential with mean 1/rate.  Prints one JSON
line per rate with p50 / p99 job latency and throughput.
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch

from . import _lib
from . import datasets as D
from .ops import GridSpec
from .serving import JobData, Server, poisson_load


def make_observation(rng, max_vis: float):
    G = int(rng.choice([1024, 2048, 4096, 8192]))
    ns = int(rng.integers(16, 201))
    C = int(rng.integers(8, 65))
    T = int(rng.integers(1, 33)) * 64
    nb = ns * (ns - 1) // 2
    T = int(max(64, min(T, (max_vis // (nb * C)) // 64 * 64)))
    spec = D.ObservationSpec(nstations=ns, disk_radius_m=5000.0 * G / 4096, ntimesteps=T, timesteps_per_subgrid=64,
                             nchannels=C, f_start=150e6, f_end=160e6, subgrid_size=32, grid_size=G, image_size=0.05,
                             aterm_sigma=0.05, aterm_interval=256, seed=int(rng.integers(1 << 30)))
    obs = D.make_observation(spec)
    gs = GridSpec(G, 32, C, ns, obs.aterms.shape[0], 1, spec.image_size)
    vis = D.visibilities(spec, device="cuda", seed=spec.seed)
    vis_host = torch.empty(vis.shape, dtype=vis.dtype, pin_memory=True)
    vis_host.copy_(vis)
    out_host = torch.zeros_like(vis_host).pin_memory()
    # every host input page-locked, as a serving client keeps them: a copy from
    # pageable memory runs through a staging buffer at the host's pageable rate
    # and holds the server's scheduler thread meanwhile
    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()

    uvw, k, taper, aterms = pinned(obs.uvw), pinned(obs.wavenumbers), pinned(obs.taper), pinned(obs.aterms)
    grid_job = JobData(gs, obs.metadata, uvw, k, taper, aterms, vis_host)
    degrid_job = JobData(gs, obs.metadata, uvw, k, taper, aterms, out_host)
    return spec, grid_job, degrid_job


def host_copy_gbs(observations, repeats: int = 3) -> dict:
    """Copy rates (GB/s) of the jobs' page-locked visibility buffers just before
    a stream: the first observation's input array to the device and back,
    `repeats` times each way, best taken.  Job latencies include these copies,
    so the serving line carries the rate they ran at."""
    src = observations[0][1].vis
    dev = torch.empty_like(src, device="cuda")
    rates = {}
    for name, dst, frm in (("h2d_gbs", dev, src), ("d2h_gbs", src, dev)):
        best = 0.0
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(frm, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = max(best, src.numel() * src.element_size() / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        rates[name] = round(best, 1)
    del dev
    return rates


def run_stream(observations, rate: float, slots: int = 4, budget_gb: float = 96.0, seed: int = 5) -> dict:
    """Serve the gridding and degridding jobs of `observations` as one Poisson
    stream of mean rate `rate` jobs/s; returns the latency / throughput line.
    One gridding and one degridding job of the first observation run before
    the stream (into a grid of their own) so that the server's one-time set-up
    is not timed; the percentiles are over the stream's jobs (linear
    interpolation between order statistics)."""
    copy_rates = host_copy_gbs(observations)
    with Server(max_slots=slots, hbm_budget_bytes=int(budget_gb * (1 << 30)), cta_share=True) as srv:
        spec0, gjob0, djob0 = observations[0]
        warm = srv.grid_create(spec0.grid_size)
        srv.wait(srv.submit(_lib.IDG_JOB_GRID, gjob0, warm))
        srv.wait(srv.submit(_lib.IDG_JOB_DEGRID, djob0, warm))
        srv.grid_release(warm)
        grids = [srv.grid_create(spec.grid_size) for spec, _, _ in observations]
        # a random interleaving in which each observation's gridding job precedes its degridding job
        order = np.random.default_rng(seed + 1).permutation(2 * len(observations)).reshape(-1, 2)
        events = []
        for i, (p, q) in enumerate(order):
            events.append((min(p, q), (_lib.IDG_JOB_GRID, observations[i][1], grids[i])))
            events.append((max(p, q), (_lib.IDG_JOB_DEGRID, observations[i][2], grids[i])))
        stream = [job for _, job in sorted(events, key=lambda e: e[0])]
        st = poisson_load(srv, stream, rate, seed=seed)
        for g in grids:
            srv.grid_release(g)
    lat = sorted(j["latency_ms"] for j in st["jobs"])
    nvis = int(sum(j["visibilities"] for j in st["jobs"]))
    return {
        "metric": "serving: job latency and throughput, Poisson arrivals",
        "rate_jobs_per_s": rate,
        "jobs": len(stream),
        "completed": st["completed"] - 2,
        "rejected": st["rejected"],
        "p50_ms": float(np.percentile(lat, 50)) if lat else None,
        "p99_ms": float(np.percentile(lat, 99)) if lat else None,
        "mean_ms": float(np.mean(lat)) if lat else None,
        "max_ms": lat[-1] if lat else None,
        "mvis_per_s": nvis / st["wall_s"] / 1e6,
        "warmup_jobs": 2,
        "hbm_peak_gb": st["hbm_peak"] / 1e9,
        "slots": slots,
        "budget_gb": budget_gb,
        "visibilities": nvis,
        "wall_s": st["wall_s"],
        "host_copy_gbs": copy_rates,
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="2,4,8")
    ap.add_argument("--jobs", type=int, default=24, help="observations per rate (each gives 2 jobs)")
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--budget-gb", type=float, default=96.0)
    ap.add_argument("--max-vis", type=float, default=1.3e8)
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args(argv)
    torch.cuda.init()
    rng = np.random.default_rng(args.seed)
    observations = [make_observation(rng, args.max_vis) for _ in range(args.jobs)]
    results = []
    for rate in [float(r) for r in args.rates.split(",")]:
        line = run_stream(observations, rate, args.slots, args.budget_gb, args.seed)
        print(json.dumps(line), flush=True)
        results.append(line)
    return results


if __name__ == "__main__":
    main()
