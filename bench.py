#!/usr/bin/env python3
"""IDG grid + degrid throughput on one GB300 (or N independent ones).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config2|config1] [--variant batched|plain]

A step is one imaging cycle over the whole workload: the gridding step
(gridder -> subgrid FFT -> adder into the uv-grid) followed by the degridding
step (splitter -> subgrid FFT -> degridder back into visibilities).  The
default workload is the 100-station / 4950-baseline / 8192 x 1 s / 16-channel
/ 32x32-subgrid / 4096^2-grid observation (316,800 subgrids, 6.49e8
visibilities, 20.8 GB of visibilities), seeded synthetic data.

Printed (rank 0, one JSON line):
  value   Mvis/s = visibilities / (device time of one step), inputs resident in HBM
  e2e     the same through the C ABI on page-locked host buffers, with every
          step's copies in (plan, uvw, visibilities) and out (visibilities)
          inside the timed region: the K steps are K cycles of one
          idg_imaging_cycles() call, each cycle's copies in running while the
          cycle before it degrids; `single_cycle` beside it is one
          idg_imaging_cycle() call per step
  roofline of the gridder and the degridder: 17 FMA (34 flop) per
          pixel-visibility over the measured FP32 FMA peak of this device; the
          top-level figures are those of the kernel with the larger time share
  cpu_baseline the reference's CPU algorithm (the oracle's float restatement of
          its OpenMP launchers) on a bounded sample of the same workload
  serving p50 / p99 job latency and Mvis/s of a Poisson stream of gridding and
          degridding jobs of mixed sizes (16-200 stations, 64-2048 timesteps,
          8-64 channels, 1024^2-8192^2 grids) served with continuous batching
  imaging the uv-grid -> image FFT of the cycle's grid (idg_grid_fft), timed
          separately, with its HBM rate

--impl reference times that CPU implementation alone (rank 0) on the same
workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ska-spc-tender-benchmarks_gb300"))

METRIC = "Mvis/s grid+degrid vs plain GPU form at ≤1e-5 rel err; p50/p99 job latency"
FLOP_PER_PIXVIS = 34.0  # 16 FMA of the four complex MACs + 1 FMA of the phase
# DRAM bytes (read + write) per subgrid of one batched kernel launch, S = 32, 16
# channels x 128 timesteps: ncu capture of one launch on the first 8192
# subgrids of the config-2 plan with the tuned mirror-quad shapes (gridder
# shape 24: 690.4 MB read + 245.2 MB written; degridder shape 34: 418.4 MB
# read + 490.1 MB written), divided by 8192.
DRAM_BYTES_PER_SUBGRID = {"gridder": 114213.0, "degridder": 110901.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["config2", "config1"], default="config2")
    ap.add_argument("--variant", choices=["batched", "plain"], default="batched")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of each baseline half")
    ap.add_argument("--skip-cpu", action="store_true", help="no CPU baseline (profiling runs)")
    ap.add_argument("--max-subgrids", type=int, default=0, help="use only the first N subgrids of the plan (profiling)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving (p50/p99 latency) leg")
    ap.add_argument("--serve-jobs", type=int, default=30, help="observations in the serving leg (2 jobs each)")
    ap.add_argument("--serve-rates", default="4,16,32", help="mean arrival rates of the serving leg, jobs/s")
    ap.add_argument("--no-uneven", action="store_true", help="skip the batched-uneven (50,000 mixed subgrids) leg")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="reference arm: skip timing the reference's own CUDA kernels")
    ap.add_argument("--shapes", default="", help="G,D: batched gridder/degridder launch shapes instead of autotuning")
    ap.add_argument("--host-buffers", choices=["auto", "pinned", "hostmem"], default="auto",
                    help="page-locked host buffers of the e2e leg: cudaHostAlloc (pinned), huge-page memory "
                         "registered with cudaHostRegister (hostmem), or whichever runs a trial imaging cycle faster (auto)")
    return ap.parse_args()


def workload_spec(name: str, seed: int):
    from idg_gb300 import datasets as D

    return D.config2(seed=seed) if name == "config2" else D.config1(seed=seed)


def host_mem_available() -> int:
    """MemAvailable of this host in bytes (a large value when it cannot be read)."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 1 << 50


def e2e_prefix(metadata: np.ndarray, n_rows: int, bytes_per_row: int, budget: float) -> tuple[int, int]:
    """(subgrids, rows) of the e2e leg: the whole plan when n_rows rows of
    bytes_per_row fit in budget, else the leading subgrids whose rows fit
    (at least one subgrid)."""
    rows_fit = int(budget // bytes_per_row)
    if rows_fit >= n_rows:
        return metadata.shape[0], n_rows
    row_end = metadata["time_offset"].astype(np.int64) + metadata["nr_timesteps"]
    n = max(1, int(np.searchsorted(np.maximum.accumulate(row_end), rows_fit, side="right")))
    return n, int(row_end[:n].max())


def config_block(spec, name, extra=None):
    c = {
        "workload": f"{name}: {spec.nstations} stations in a {2 * spec.disk_radius_m / 1000:g} km disk, "
                    f"{spec.n_baselines} baselines x {spec.ntimesteps} x {spec.integration_s:g} s in "
                    f"{spec.timesteps_per_subgrid}-step subgrids, {spec.nchannels} channels "
                    f"{spec.f_start / 1e6:g}-{spec.f_end / 1e6:g} MHz, subgrid {spec.subgrid_size}^2, "
                    f"grid {spec.grid_size}^2, image size {spec.image_size} rad",
        "n_subgrids": spec.n_subgrids,
        "n_visibilities": spec.n_visibilities,
        "subgrid_size": spec.subgrid_size,
        "grid_size": spec.grid_size,
        "nchannels": spec.nchannels,
        "l2": "inputs larger than L2 (visibilities %.1f GB)" % (spec.n_rows * spec.nchannels * 32 / 1e9),
    }
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# CPU baseline: the reference's CPU algorithm on a bounded sample
# ---------------------------------------------------------------------------
def cpu_baseline(obs, vis_host: np.ndarray, target_s: float, build: str = "-O2"):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build(with_ref=False)
    spec = obs.spec
    S, C, T = spec.subgrid_size, spec.nchannels, spec.timesteps_per_subgrid
    md_all = obs.metadata

    # the sample may only use subgrids whose rows are all in vis_host
    row_end = md_all["time_offset"].astype(np.int64) + md_all["nr_timesteps"]
    n_avail = int(np.searchsorted(np.maximum.accumulate(row_end), vis_host.shape[0], side="right"))
    if n_avail < 1:
        raise ValueError("cpu_baseline: vis_host holds no complete subgrid")

    def run(n, grid_too=True):
        md = md_all[:n].copy()
        rows = int(md["time_offset"][-1] + md["nr_timesteps"][-1])
        if rows > vis_host.shape[0]:
            raise ValueError(f"cpu_baseline: sample of {n} subgrids needs {rows} rows, vis_host has {vis_host.shape[0]}")
        prm = O.params(spec.grid_size, S, C, spec.nstations, n, spec.image_size)
        uvw = np.ascontiguousarray(obs.uvw[:rows])
        vis = np.ascontiguousarray(vis_host[:rows])
        sub = np.zeros((n, 4, S, S), np.complex64)
        t0 = time.perf_counter()
        O.cpu_gridding_omp(prm, uvw, obs.wavenumbers, vis, obs.taper, np.ascontiguousarray(obs.aterms), md, sub,
                           build=build)
        tg = time.perf_counter() - t0
        out = np.zeros_like(vis)
        t0 = time.perf_counter()
        O.cpu_degridding_omp(prm, uvw, obs.wavenumbers, sub, obs.taper, np.ascontiguousarray(obs.aterms), md, out,
                             build=build)
        td = time.perf_counter() - t0
        return tg, td

    n = min(8, n_avail)
    tg, td = run(n)
    per = max((tg + td) / n, 1e-6)
    n = int(max(min(8, n_avail), min(n_avail, (2 * target_s) / per)))
    tg, td = run(n)
    nvis = n * T * C
    return {
        "value": nvis / (tg + td) / 1e6,
        "unit": "Mvis/s",
        "cores": O.omp_threads(),
        "kind": "port",
        "sample": f"first {n} of {spec.n_subgrids} subgrids of the same plan ({nvis} visibilities); "
                  f"gridding {tg:.2f} s + degridding {td:.2f} s on {O.omp_threads()} OpenMP threads "
                  f"(float restatement of the reference's OpenMP CPU launchers, {build})",
    }


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# host buffers of the e2e leg
# ---------------------------------------------------------------------------
def copy_probe(host_in, host_out, dev_buf, stream, chunks=32) -> dict:
    """Plain cudaMemcpyAsync rates (GB/s) between two page-locked host arrays
    and a device buffer of the same size: the whole array in `chunks` copies,
    host to device, then device to host, each timed with CUDA events."""
    import torch

    hi = torch.from_numpy(host_in).view(torch.uint8).reshape(-1)
    ho = torch.from_numpy(host_out).view(torch.uint8).reshape(-1)
    d = dev_buf.view(torch.uint8).reshape(-1)
    n = min(hi.numel(), d.numel())
    step = max(1, n // chunks)
    rates = {}
    for direction in ("h2d", "d2h"):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for c0 in range(0, n, step):
                sl = slice(c0, min(n, c0 + step))
                if direction == "h2d":
                    d[sl].copy_(hi[sl], non_blocking=True)
                else:
                    ho[sl].copy_(d[sl], non_blocking=True)
            e1.record(stream)
        e1.synchronize()
        rates[direction + "_gbs"] = round(n / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
    return rates


def e2e_host_buffers(kind: str, shape, fill, dev_buf, stream):
    """The e2e leg's candidate input and output visibility arrays, page-locked.

    "pinned": cudaHostAlloc (torch pin_memory); "hostmem": transparent-huge-
    page memory registered with cudaHostRegister (idg_gb300.hostmem); "auto":
    both, where host memory allows, and the caller keeps the kind whose
    imaging cycle runs faster.  The two kinds copy at the same rate on a
    healthy host (about 210 GB/s in, 190 GB/s out on GB300), but cudaHostAlloc
    memory has been measured well below its own copy probe inside the cycle
    (39 GB/s in against a 137 GB/s probe), so the choice rests on a cycle and
    not on the probe.  Returns (candidates, record): candidates maps each kind
    made to its (vis_in, vis_out) pair; the record holds every probe taken."""
    import torch

    from idg_gb300 import hostmem

    def make(k):
        if k == "pinned":
            a = torch.empty(shape, dtype=torch.complex64, pin_memory=True).numpy()
            b = torch.empty(shape, dtype=torch.complex64, pin_memory=True).numpy()
        else:
            a = hostmem.pinned_empty(shape, np.complex64)
            b = hostmem.pinned_empty(shape, np.complex64)
        torch.from_numpy(a).copy_(fill)
        copy_probe(a, b, dev_buf, stream)  # first touch of the pages by the copy engines
        return a, b, copy_probe(a, b, dev_buf, stream)

    kinds = ["hostmem", "pinned"] if kind == "auto" else [kind]
    cands, probes = {}, {}
    for k in kinds:
        if cands and host_mem_available() < 1.5 * sum(x.nbytes for x in next(iter(cands.values()))):
            break
        a, b, pr = make(k)
        cands[k] = (a, b)
        probes[k] = pr
    return cands, {"kind": next(iter(cands)), "probes": probes}


def release_host_buffers(record, *arrays):
    """Unregisters host arrays of the record's kind when they are hostmem
    arrays (the memory goes with the last reference)."""
    from idg_gb300 import hostmem

    if record["kind"] == "hostmem":
        for a in arrays:
            hostmem.release(a)


def free_pinned_cache():
    """Returns torch's cached page-locked host blocks that no array holds any
    more (pinned arrays stay in its cache after their last reference)."""
    import gc

    import torch

    gc.collect()
    if hasattr(torch._C, "_host_emptyCache"):
        torch._C._host_emptyCache()


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank):
    import torch

    from idg_gb300 import datasets as D
    from idg_gb300 import hostmem, ops

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    spec = workload_spec(args.workload, seed=2 if args.workload == "config2" else 1)
    obs = D.make_observation(spec)
    if args.max_subgrids:
        obs = D.truncate_observation(obs, args.max_subgrids)
        spec = obs.spec
    S, C, G = spec.subgrid_size, spec.nchannels, spec.grid_size
    N = spec.n_subgrids
    gs = ops.GridSpec(G, S, C, spec.nstations, obs.aterms.shape[0], 1, spec.image_size, spec.w_step)
    variant = ops.VARIANT_BATCHED if args.variant == "batched" else ops.VARIANT_PLAIN

    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        md = ops.metadata_tensor(obs.metadata, dev)
        uvw = torch.from_numpy(obs.uvw).to(dev)
        k = torch.from_numpy(obs.wavenumbers).to(dev)
        taper = torch.from_numpy(obs.taper).to(dev)
        at = torch.from_numpy(obs.aterms).to(dev)
        vis = D.visibilities(spec, device=dev, seed=spec.seed + 1000 * rank)
        vis_out = torch.empty_like(vis)
        sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device=dev)
        grid = torch.empty((1, 4, G, G), dtype=torch.complex64, device=dev)
    stream.synchronize()

    nogrid = gs.__class__(**{**gs.__dict__, "flags": gs.flags | 0x2})  # IDG_FLAG_NO_TAPER
    # the adder with a fixed summation order, as the plan's cycle runs it
    bins = ops.TileBins(gs, obs.metadata)

    # autotune the batched kernels' launch shapes on a leading sample of the plan
    tune = None
    if variant == ops.VARIANT_BATCHED and args.shapes:
        from idg_gb300 import tuning

        gsh, dsh = (int(x) for x in args.shapes.split(","))
        tuning.set_shapes(S, gsh, dsh)
        tune = {"gridder": gsh, "degridder": dsh, "fixed": True}
    elif variant == ops.VARIANT_BATCHED:
        from idg_gb300 import tuning

        ns = min(N, 8192)
        rows_s = int(obs.metadata["time_offset"][ns - 1] + obs.metadata["nr_timesteps"][ns - 1])
        tune = tuning.autotune(nogrid, md[:ns], uvw[:rows_s], k, vis[:rows_s], None, at, sub[:ns], vis_out[:rows_s],
                               repeats=2, stream=stream, store=False)

    # e2e through the host-buffer cycles on page-locked host buffers, with the tuned
    # shapes, before the device-resident legs.  Every rank locks its
    # visibilities in and out; when the ranks of this node would not fit in
    # the host memory available, the e2e leg uses the leading subgrids that do
    # (and says so), instead of failing.  The host buffers' copy rate is probed
    # (plain cudaMemcpyAsync, the visibilities in 32 chunks each way) just
    # before the leg, and each cycle reports the rate its own copies ran at.
    e2e = None
    cpu = None
    vis_host = None
    small = []  # page-locked plan, uvw and A-terms of the e2e leg
    host_rec = None
    local_world = int(os.environ.get("LOCAL_WORLD_SIZE", world))
    e2e_n, e2e_rows = e2e_prefix(obs.metadata, spec.n_rows, 2 * C * 32,
                                 0.6 * host_mem_available() / max(1, local_world))
    if not args.no_e2e:
        cands, host_rec = e2e_host_buffers(args.host_buffers, (e2e_rows,) + tuple(vis.shape[1:]),
                                           vis[:e2e_rows], vis_out[:e2e_rows], stream)
        chunk = -2  # IDG_CHUNKS_ADAPTIVE: gridding chunks growing (ratio from the last cycle), degridding shrinking
        aterms_np = hostmem.pinned_copy(obs.aterms)
        md_e2e = hostmem.pinned_copy(obs.metadata[:e2e_n])
        uvw_e2e = hostmem.pinned_copy(obs.uvw[:e2e_rows])
        small = [aterms_np, md_e2e, uvw_e2e]
        nvis_e2e = int(md_e2e["nr_timesteps"].astype(np.int64).sum()) * C

        def cycle(pair):
            return ops.imaging_cycle(gs, md_e2e, uvw_e2e, obs.wavenumbers, pair[0], obs.taper, aterms_np, pair[1],
                                     variant=variant, chunk_subgrids=chunk)

        cycle(next(iter(cands.values())))  # warm: allocates the cycle's device buffers
        trial = {}
        for kind, pair in cands.items():  # one cycle per kind of host buffer; the faster one is kept
            t = cycle(pair)
            trial[kind] = {"ms": round(float(t["total_ms"]), 1),
                           "h2d_gbs": round(t["h2d_vis_bytes"] / (t["h2d_vis_ms"] * 1e-3) / 1e9, 1)}
        best = min(trial, key=lambda kd: trial[kd]["ms"])
        for kind in [kd for kd in cands if kd != best]:
            pair = cands.pop(kind)
            release_host_buffers({"kind": kind}, *pair)
            del pair
            free_pinned_cache()
        vis_host, out_host = cands.pop(best)
        host_rec["kind"] = best
        cycle((vis_host, out_host))

        def gbs(t, d):
            return round(t[d + "_vis_bytes"] / (t[d + "_vis_ms"] * 1e-3) / 1e9, 1)

        # one cycle per call (idg_imaging_cycle): its copies in all fall in
        # its own gridding phase
        singles = [cycle((vis_host, out_host)) for _ in range(min(args.steps, 5))]
        single_ms = float(np.mean([t["total_ms"] for t in singles]))
        # the timed steps: K cycles in one idg_imaging_cycles call, each
        # copying its plan, uvw and visibilities in (during the degridding of
        # the cycle before it) and its visibilities out
        run = [(md_e2e, uvw_e2e, vis_host, out_host)]
        ops.imaging_cycles(gs, run * 2, obs.wavenumbers, obs.taper, aterms_np, variant=variant,
                           chunk_subgrids=chunk)  # warm: the second plan / uvw buffers
        if dist:
            dist.barrier()
        w0 = time.perf_counter()
        totals = ops.imaging_cycles(gs, run * args.steps, obs.wavenumbers, obs.taper, aterms_np, variant=variant,
                                    chunk_subgrids=chunk)
        wall_ms = (time.perf_counter() - w0) * 1e3
        ends = [float(t["end_ms"]) for t in totals]
        e2e_ms = ends[-1] / args.steps
        if dist:
            tt = torch.tensor([e2e_ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_ms = float(tt.item())
        steps_ms = [ends[0]] + [b - a for a, b in zip(ends, ends[1:])]
        e2e = {"value": world * nvis_e2e / (e2e_ms * 1e-3) / 1e6, "unit": "Mvis/s",
               "h2d_bytes_per_step": int(np.mean([t["h2d_bytes"] for t in totals])),
               "d2h_bytes_per_step": int(np.mean([t["d2h_bytes"] for t in totals])),
               "ms_per_step": e2e_ms,
               "api": "idg_imaging_cycles (C ABI) on page-locked host buffers: the K timed steps are K cycles of one "
                      "call, each copying its inputs in and its visibilities out; a cycle's copies in run during "
                      "the degridding of the cycle before it",
               "timed_from": "the first cycle's first copy in to the last cycle's last copy out (CUDA events)",
               "host_wall_ms_per_step": round(wall_ms / args.steps, 1),
               "first_step_h2d_bytes": int(totals[0]["h2d_bytes"]),
               "host_buffers": host_rec["kind"],
               "host_buffer_trial": trial,
               "copy_probe_gbs": host_rec["probes"],
               "h2d_gbs_steps": [gbs(t, "h2d") for t in totals],
               "d2h_gbs_steps": [gbs(t, "d2h") for t in totals],
               "host_buffers_gb": round((vis_host.nbytes + out_host.nbytes + sum(x.nbytes for x in small)) / 1e9, 2),
               "subgrids": e2e_n,
               "chunks": {"gridding": int(totals[-1]["grid_chunks"]), "degridding": int(totals[-1]["degrid_chunks"])},
               "chunk_ratio": round(totals[0]["chunk_ratio"], 3),
               "gridding_wait_ms_steps": [round(t["gridding_wait_ms"], 1) for t in totals],
               "h2d_ms_steps": [round(t["h2d_vis_ms"], 1) for t in totals],
               "h2d_span_ms_steps": [round(t["h2d_span_ms"], 1) for t in totals],
               "gridding_ms": float(np.mean([t["gridding_ms"] for t in totals])),
               "degridding_ms": float(np.mean([t["degridding_ms"] for t in totals])),
               "steps_ms": [round(x, 1) for x in steps_ms],
               "steps_spread": round((max(steps_ms) - min(steps_ms)) / e2e_ms, 4),
               "single_cycle": {"api": "idg_imaging_cycle, one cycle per call",
                                "value": world * nvis_e2e / (single_ms * 1e-3) / 1e6,
                                "ms_per_step": single_ms, "steps": len(singles),
                                "steps_ms": [round(t["total_ms"], 1) for t in singles],
                                "h2d_gbs_steps": [gbs(t, "h2d") for t in singles],
                                "chunk_ratio_steps": [round(t["chunk_ratio"], 3) for t in singles],
                                "gridding_wait_ms_steps": [round(t["gridding_wait_ms"], 1) for t in singles],
                                "gridding_ms_steps": [round(t["gridding_ms"], 1) for t in singles],
                                "h2d_ms_steps": [round(t["h2d_vis_ms"], 1) for t in singles],
                                "h2d_span_ms_steps": [round(t["h2d_span_ms"], 1) for t in singles]}}
        # free the cycle's device buffers and the e2e inputs (vis_host stays for the CPU baseline)
        ops.release_buffers()
        for a in small:
            hostmem.release(a)
        release_host_buffers(host_rec, out_host)
        del out_host, aterms_np, md_e2e, uvw_e2e, small
        free_pinned_cache()
    elif rank == 0 and not args.skip_cpu:
        vis_host = vis[:e2e_rows].cpu().numpy()

    def step(v=variant, ev=None):
        # gridding step
        grid.zero_()
        if ev: ev[0].record(stream)
        ops.gridder(nogrid, md, uvw, k, vis, None, at, sub, variant=v, stream=stream)
        if ev: ev[1].record(stream)
        ops.subgrid_fft(gs, sub, +1, taper, stream=stream)
        if ev: ev[2].record(stream)
        bins.add(sub, grid, stream=stream)
        if ev: ev[3].record(stream)
        # degridding step: splitter and backward FFT in one pass, then the degridder
        ops.split_subgrid_fft(gs, md, grid, sub, taper, stream=stream)
        if ev: ev[4].record(stream)
        ops.degridder(nogrid, md, uvw, k, vis_out, None, at, sub, variant=v, stream=stream)
        if ev: ev[5].record(stream)

    # The batched form runs as one captured CUDA graph per cycle over a device-resident
    # plan (longest-first work list, tuned launch shapes); the plain form as direct calls.
    plan = None
    if variant == ops.VARIANT_BATCHED:
        plan = ops.Plan(gs, obs.metadata, spec.n_rows, variant=ops.VARIANT_BATCHED)
        plan.capture_cycle(uvw, k, vis, taper, at, grid, vis_out)

    def cycle():
        if plan is not None:
            plan.launch_cycle(stream)
        else:
            step()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            cycle()
    stream.synchronize()
    if ops.device_status(clear=True) or (plan is not None and plan.status()):
        raise RuntimeError("a kernel rejected plan entries during warm-up")

    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        t0.record(stream)
        for i in range(args.steps):
            cycle()
        t1.record(stream)
    t1.synchronize()
    torch.cuda.synchronize(dev)
    clock_info = clocks.stop()
    if dist:
        dist.barrier()
    elapsed_ms = t0.elapsed_time(t1)
    if dist:
        tt = torch.tensor([elapsed_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        elapsed_ms = float(tt.item())
    ms_per_step = elapsed_ms / args.steps
    nvis = spec.n_visibilities
    value = world * nvis / (ms_per_step * 1e-3) / 1e6

    # per-kernel times of the same kernels (direct calls, events between launches)
    # for the roofline: one instrumented cycle after the timed region
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    with torch.cuda.stream(stream):
        step(ev=ev)
    stream.synchronize()
    parts = np.array([[ev[j].elapsed_time(ev[j + 1]) for j in range(5)]])

    # roofline (FP32 FMA bound) of the gridder and the degridder; the JSON's
    # top-level figures are those of the kernel with the larger time share
    pixvis = float(nvis) * S * S
    grid_ms = float(np.mean(parts[:, 0]))
    degrid_ms = float(np.mean(parts[:, 4]))
    peak = ops.measure_fp32_peak()
    per_kernel = {}
    for name, ms in (("gridder", grid_ms), ("degridder", degrid_ms)):
        ach = FLOP_PER_PIXVIS * pixvis / (ms * 1e-3)
        traffic = DRAM_BYTES_PER_SUBGRID[name] * N if S == 32 else None
        per_kernel[name] = {"achieved": ach / 1e12, "frac": ach / peak, "ms": ms, "traffic": traffic}
    dom = "degridder" if degrid_ms > grid_ms else "gridder"
    # the measured FFMA peak against 128 FP32 lanes x 2 flop per SM clock, at
    # the SM clock sampled over the timed region (the microbenchmark itself
    # runs for milliseconds, below the sampler's 200 ms period)
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = clock_info["sm_mhz"] if clock_info else None
    theory = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6 if sm_mhz else None
    peak_check = {"sms": props.multi_processor_count, "fp32_lanes_per_sm": 128, "sm_mhz": sm_mhz,
                  "lanes_x_2_x_clock_tflops": theory / 1e12 if theory else None,
                  "measured_over_lanes_x_2_x_clock": peak / theory if theory else None}
    roof = {
        "bound": "fp32",
        "kernel": dom,
        "achieved": per_kernel[dom]["achieved"],
        "peak": peak / 1e12,
        "unit": "TFLOP/s",
        "frac": per_kernel[dom]["frac"],
        "traffic": per_kernel[dom]["traffic"],
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the first 8192 "
                          "subgrids of this plan, scaled by subgrids (the kernels stream each subgrid's data once)",
        "peak_source": "measured in this run: FFMA microbenchmark idg_measure_fp32_peak (MEASURED_PEAKS.json "
                       "carries HBM and bf16 figures, no FP32 FMA figure); the SFU bound (16 sin/cos per SM clock, 2 per "
                       "pixel-visibility) is within 2% of the FMA bound on GB300",
        "algorithmic": "34 flop (17 FMA) + 1 sincos per pixel-visibility; %.3g pixel-visibilities per launch" % pixvis,
        "peak_check": peak_check,
        "gridder": per_kernel["gridder"],
        "degridder": per_kernel["degridder"],
        "kernel_ms": {n: float(np.mean(parts[:, j])) for j, n in enumerate(
            ["gridder", "fft_fwd", "adder", "split_fft_bwd", "degridder"])},
    }
    if plan is not None:
        plan.close()

    # imaging step around the cycle: the uv-grid -> image FFT (idg_grid_fft) on
    # this grid, outside the timed cycle; 4 HBM passes (2 row FFTs, 2 transposes)
    imaging = None
    if G <= 8192 and (G & (G - 1)) == 0:
        ge = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        with torch.cuda.stream(stream):
            ops.grid_fft(gs, grid, -1, stream=stream)  # warm (twiddle table)
            ge[0].record(stream)
            for _ in range(3):
                ops.grid_fft(gs, grid, -1, stream=stream)
            ge[1].record(stream)
        stream.synchronize()
        fft_ms = ge[0].elapsed_time(ge[1]) / 3
        nbytes = 4 * 2 * grid.numel() * 8
        hbm_peak = None
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                hbm_peak = float(json.load(f)["hbm_gbs"])
        except (OSError, ValueError, KeyError):
            pass
        ach = nbytes / (fft_ms * 1e-3) / 1e9
        imaging = {"grid_fft_ms": fft_ms, "grid": f"1x4x{G}^2",
                   "hbm_bytes": nbytes, "achieved_gbs": ach,
                   "frac_of_measured_hbm": ach / hbm_peak if hbm_peak else None,
                   "note": "not part of the timed cycle; HBM bytes = 4 passes x (read + write) of the grid"}

    # plain form (one step, same data) for the batched / plain ratio
    plain = None
    if not args.no_plain and variant != ops.VARIANT_PLAIN:
        with torch.cuda.stream(stream):
            step(v=ops.VARIANT_PLAIN)
            pe = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
            step(v=ops.VARIANT_PLAIN, ev=pe)
        stream.synchronize()
        pms = pe[0].elapsed_time(pe[5])
        plain = {"value": nvis / (pms * 1e-3) / 1e6, "unit": "Mvis/s", "ms_per_step": pms,
                 "gridder_ms": pe[0].elapsed_time(pe[1]), "degridder_ms": pe[4].elapsed_time(pe[5])}

    # serving: Poisson streams of gridding and degridding jobs of mixed sizes,
    # one per arrival rate, over the same observations
    serving = None
    if not args.no_serve:
        from idg_gb300 import serve_bench

        srng = np.random.default_rng(5 + rank)
        jobs = [serve_bench.make_observation(srng, 2e7) for _ in range(args.serve_jobs)]
        serving = [serve_bench.run_stream(jobs, float(r), slots=4, budget_gb=64.0, seed=5 + rank)
                   for r in args.serve_rates.split(",")]
        del jobs

    # batched uneven: 50,000 subgrids of mixed size, time span and channel
    # group, one CUDA graph per cycle, against the plain kernels
    uneven = None
    if not args.no_uneven and world == 1:
        from idg_gb300 import uneven_bench

        del sub, vis_out  # room for the job's own buffers
        torch.cuda.empty_cache()
        uneven = uneven_bench.run(uneven_bench.parse(["--steps", "3", "--warmup", "3"]))

    if rank == 0 and not args.skip_cpu:
        cpu = cpu_baseline(obs, vis_host, args.cpu_seconds)
    if host_rec is not None:
        release_host_buffers(host_rec, vis_host)
    del vis_host

    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return None
    return {
        "metric": METRIC,
        "value": value,
        "unit": "Mvis/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (FP64 per-subgrid phase offsets)",
        "data": "synthetic (seeded; N(0,1) visibilities, earth-rotation uvw)",
        "config": config_block(spec, args.workload, {"variant": args.variant, "parallelism": f"replicas x{world}",
                                                     "tuned_shapes": tune}),
        "e2e": e2e,
        "gpu_launches": 6 * args.steps,
        "roofline": roof,
        "cpu_baseline": cpu,
        "plain": plain,
        "serving": serving,
        "uneven": uneven,
        "imaging": imaging,
        "clocks": clock_info,
    }


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU algorithm on host cores
# ---------------------------------------------------------------------------
def reference_gpu_leg(spec, obs, steps: int = 2) -> dict:
    """The reference's own CUDA kernels, kernel_gridder_v7 and kernel_degridder_v6,
    compiled unmodified from its sources for sm_103a (oracle/_ref cubins), on the
    same workload: one launch each over the whole plan (one CTA of 128 threads
    per subgrid, as the reference launches them), device time from CUDA events,
    and their error against the FP64 oracle on 24 subgrids of short, middle
    and long baselines (the degridder against the oracle with the GPU kernel's
    own w-offset, (z + 1/2) 2 pi: degridding_benchmark.cu:33)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu

    why = ref_gpu.available()
    if why:
        return {"unavailable": why}
    import torch

    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    import oracle as O
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    S, C, G, N = spec.subgrid_size, spec.nchannels, spec.grid_size, spec.n_subgrids
    nat = obs.aterms.shape[0]
    md = ops.metadata_tensor(obs.metadata, dev)
    uvw = torch.from_numpy(obs.uvw).to(dev)
    k = torch.from_numpy(obs.wavenumbers).to(dev)
    taper = torch.from_numpy(obs.taper).to(dev)
    at = torch.from_numpy(np.ascontiguousarray(obs.aterms)).to(dev)
    vis = D.visibilities(spec, device=dev, seed=spec.seed)
    vout = torch.empty_like(vis)
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device=dev)
    torch.cuda.synchronize()
    try:
        ref_gpu.RefKernels.check_plan(obs.metadata, spec.n_rows, spec.nstations, nat, S, degridder=True)
    except ValueError as e:
        return {"unavailable": f"outside the reference kernels' safe limits: {e}"}
    K = ref_gpu.RefKernels()
    stream = torch.cuda.current_stream(dev)
    h = stream.cuda_stream
    common = dict(nr_rows=spec.n_rows, nr_aterms=nat, grid_size=G, subgrid_size=S, image_size=spec.image_size,
                  nr_channels=C, nr_stations=spec.nstations, wavenumbers=k.data_ptr(), spheroidal=taper.data_ptr(),
                  aterms=at.data_ptr(), d_metadata=md.data_ptr(), stream=h, checked=True)

    def grid():
        K.gridder(obs.metadata, uvw=uvw.data_ptr(), visibilities=vis.data_ptr(), subgrids=sub.data_ptr(), **common)

    def degrid():
        K.degridder(obs.metadata, uvw=uvw.data_ptr(), visibilities=vout.data_ptr(), subgrids=sub.data_ptr(), **common)

    grid()
    degrid()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    g_ms = d_ms = 0.0
    for _ in range(steps):
        ev[0].record(stream)
        grid()
        ev[1].record(stream)
        degrid()
        ev[2].record(stream)
        ev[2].synchronize()
        g_ms += ev[0].elapsed_time(ev[1]) / steps
        d_ms += ev[1].elapsed_time(ev[2]) / steps
    del vis, vout, sub
    torch.cuda.empty_cache()

    # error against the FP64 oracle: the first subgrid of 8 short, 8 middle and 8 long baselines
    bl_len = np.linalg.norm(obs.uvw[:: spec.ntimesteps, :2], axis=1)
    order = np.argsort(bl_len)
    pick_bl = np.concatenate([order[:8], order[len(order) // 2: len(order) // 2 + 8], order[-8:]])
    smd = obs.metadata[pick_bl * spec.subgrids_per_baseline].copy()
    rows = np.concatenate([np.arange(m["time_offset"], m["time_offset"] + m["nr_timesteps"]) for m in smd])
    smd["time_offset"] = np.arange(len(smd)) * spec.timesteps_per_subgrid
    suvw = np.ascontiguousarray(obs.uvw[rows])
    rng = np.random.default_rng(spec.seed + 77)
    svis = (rng.standard_normal((len(rows), C, 4)) + 1j * rng.standard_normal((len(rows), C, 4))).astype(np.complex64)
    ssub = (rng.standard_normal((len(smd), 4, S, S)) + 1j * rng.standard_normal((len(smd), 4, S, S))).astype(np.complex64)
    d_md, d_uvw = ops.metadata_tensor(smd, dev), torch.from_numpy(suvw).to(dev)
    d_vis, d_sub = torch.from_numpy(svis).to(dev), torch.from_numpy(ssub).to(dev)
    g_out = torch.empty_like(d_sub)
    v_out = torch.empty_like(d_vis)
    sc = dict(common, nr_rows=len(rows), d_metadata=d_md.data_ptr(), checked=False)
    K.gridder(smd, uvw=d_uvw.data_ptr(), visibilities=d_vis.data_ptr(), subgrids=g_out.data_ptr(), **sc)
    K.degridder(smd, uvw=d_uvw.data_ptr(), visibilities=v_out.data_ptr(), subgrids=d_sub.data_ptr(), **sc)
    torch.cuda.synchronize()
    K.close()
    prm = O.params(G, S, C, spec.nstations, len(smd), spec.image_size)
    want_g = O.gridder(prm, suvw, obs.wavenumbers, svis, obs.taper, obs.aterms, smd)
    prm_d = O.params(G, S, C, spec.nstations, len(smd), spec.image_size, 1.0)  # w-offset pi n, as the kernel
    want_v = O.degridder(prm_d, suvw, obs.wavenumbers, ssub, obs.taper, obs.aterms, smd, len(rows),
                         aterm_mode=O.ATERM_ADJOINT)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    nvis = spec.n_visibilities
    return {
        "value": nvis / ((g_ms + d_ms) * 1e-3) / 1e6,
        "unit": "Mvis/s",
        "gridder_ms": g_ms,
        "degridder_ms": d_ms,
        "steps": steps,
        "kernels": "kernel_gridder_v7 + kernel_degridder_v6 (gridding/src/gridding_benchmark.cu, "
                   "degridding_benchmark.cu) compiled unmodified for sm_103a, one CTA of 128 threads per subgrid",
        "rel_rms_vs_fp64": {"gridder": rel(g_out.cpu().numpy(), want_g), "degridder": rel(v_out.cpu().numpy(), want_v),
                            "sample": "first subgrid of 8 short, 8 middle and 8 long baselines"},
    }


def run_reference(args, rank, world):
    if rank != 0:
        return None
    from idg_gb300 import datasets as D

    spec = workload_spec(args.workload, seed=2 if args.workload == "config2" else 1)
    obs = D.make_observation(spec)
    rng = np.random.default_rng(spec.seed)
    rows = int(min(spec.n_rows, 2048 * spec.timesteps_per_subgrid))
    vis = (rng.standard_normal((rows, spec.nchannels, 4), dtype=np.float32) +
           1j * rng.standard_normal((rows, spec.nchannels, 4), dtype=np.float32)).astype(np.complex64)
    per_step = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_baseline(obs, vis, min(per_step, 3.0) / 2)
    vals = []
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(obs, vis, per_step / 2)
        vals.append(last["value"])
    value = float(np.mean(vals))
    last["value"] = value
    # the same restatement built as the reference's CMake builds it (-g, no
    # optimisation) and at -O3, each on a short bounded sample
    builds = {"-O2": value}
    for b in ("-O3", "-O0 -g"):
        builds[b] = cpu_baseline(obs, vis, 2.5, build=b)["value"]
    return {
        "metric": METRIC,
        "impl": "reference",
        "value": value,
        "unit": "Mvis/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": config_block(spec, args.workload, {"parallelism": "host cores"}),
        "cpu_baseline": last,
        "cpu_builds_mvis_per_s": builds,
        "e2e": {"value": value, "unit": "Mvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": reference_gpu_leg(spec, obs) if not args.no_ref_gpu else None,
    }


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local_rank)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
