"""Batched-uneven benchmark (config-4 generator): plain vs batched form.

    python -m idg_gb300.uneven_bench [--subgrids 50000] [--stations 2000] [--steps 3] [--warmup 3]

50,000 subgrids sampled from 2000 stations' baselines, timesteps per subgrid
log-uniform in [16, 256], channel groups of 8/16/32/64, subgrid sizes 24, 32
and 48, one 8192^2 grid (see datasets.config4).  One step is one imaging cycle
of the whole job: every size's gridding step into the shared grid, then every
size's degridding step.

* plain: the plain kernels called directly, one call sequence per size.
* batched: one plan per size (longest-first work list, autotuned launch
  shapes), the whole job captured as ONE CUDA graph (idg_cycle_capture) and
  replayed.

Prints one JSON line: Mvis/s of both forms (visibilities of the job / device
time of one step, CUDA events, inputs resident in HBM), their ratio, and the
relative RMS difference of the two forms' grids and visibilities.
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch

from . import _lib
from . import datasets as D
from . import ops, tuning


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--subgrids", type=int, default=50000)
    ap.add_argument("--stations", type=int, default=2000)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--seed", type=int, default=4)
    return ap.parse_args(argv)


def run(args) -> dict:
    """Builds the job, times both forms and returns the result line."""
    dev = torch.device("cuda")
    parts = D.config4(n_subgrids=args.subgrids, nstations=args.stations, seed=args.seed)
    G = parts[0].spec.grid_size
    stream = torch.cuda.Stream(dev)
    groups = []
    tuned = {}
    nvis = 0
    with torch.cuda.stream(stream):
        grid_p = torch.zeros((1, 4, G, G), dtype=torch.complex64, device=dev)
        grid_b = torch.zeros_like(grid_p)
        for i, o in enumerate(parts):
            S, C, N = o.spec.subgrid_size, o.spec.nchannels, o.metadata.shape[0]
            rows = o.uvw.shape[0]
            nvis += int(((o.ext["channel_end"] - o.ext["channel_begin"]) * o.metadata["nr_timesteps"]).sum())
            sp = ops.GridSpec(G, S, C, o.spec.nstations, 1, 1, o.spec.image_size)
            g = torch.Generator(device=dev)
            g.manual_seed(args.seed * 100 + i)
            vis = torch.view_as_complex(torch.randn(rows * C * 4 * 2, generator=g, device=dev).view(-1, 2)).view(rows, C, 4)
            d = dict(md=ops.metadata_tensor(o.metadata, dev), uvw=torch.from_numpy(o.uvw).to(dev),
                     k=torch.from_numpy(o.wavenumbers).to(dev), vis=vis, taper=torch.from_numpy(o.taper).to(dev),
                     at=torch.from_numpy(o.aterms).to(dev), ext=ops.ext_tensor(o.ext, dev),
                     sub=torch.empty((N, 4, S, S), dtype=torch.complex64, device=dev),
                     vout_p=torch.zeros_like(vis), vout_b=torch.zeros_like(vis))
            # autotune this size's batched shapes on a leading sample
            ns = min(N, 4096)
            r1 = int(o.metadata["time_offset"][ns - 1] + o.metadata["nr_timesteps"][ns - 1])
            res = tuning.autotune(sp, d["md"][:ns], d["uvw"][:r1], d["k"], d["vis"][:r1], d["taper"], d["at"],
                                  d["sub"][:ns], d["vout_b"][:r1], ext=d["ext"][:ns], repeats=1, stream=stream,
                                  store=False)
            tuned[S] = {"gridder": res["gridder"], "degridder": res["degridder"]}
            plan = ops.Plan(sp, o.metadata, rows, ext=o.ext, variant=_lib.VARIANT_BATCHED)
            groups.append((sp, d, plan))
    stream.synchronize()
    cyc = ops.Cycle([p for _, _, p in groups],
                    [(d["uvw"], d["k"], d["vis"], d["taper"], d["at"], d["vout_b"]) for _, d, _ in groups], grid_b)

    def plain_step():
        grid_p.zero_()
        for sp, d, _ in groups:
            ops.grid_visibilities(sp, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], d["sub"], grid_p,
                                  variant=_lib.VARIANT_PLAIN, ext=d["ext"], stream=stream)
        for sp, d, _ in groups:
            ops.degrid_visibilities(sp, d["md"], d["uvw"], d["k"], d["vout_p"], d["taper"], d["at"], d["sub"], grid_p,
                                    variant=_lib.VARIANT_PLAIN, ext=d["ext"], stream=stream)

    def timed(fn):
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                fn()
            stream.synchronize()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(args.steps):
                fn()
            t1.record(stream)
        t1.synchronize()
        return t0.elapsed_time(t1) / args.steps

    ms_b = timed(lambda: cyc.launch(stream))
    ms_p = timed(plain_step)
    for _, _, p in groups:
        if p.status():
            raise RuntimeError("a batched kernel rejected plan entries")
    rel = lambda a, b: float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    line = {
        "metric": "batched-uneven imaging cycle, Mvis/s (grid + degrid)",
        "workload": f"config4: {args.subgrids} subgrids from {args.stations} stations, T log-uniform [16, 256], "
                    f"channel groups 8/16/32/64 of 64, S in 24/32/48, grid {G}^2",
        "visibilities": nvis,
        "pixel_visibilities": float(sum(int(((o.ext["channel_end"] - o.ext["channel_begin"]).astype(np.int64) *
                                             o.metadata["nr_timesteps"]).sum()) * o.spec.subgrid_size ** 2
                                        for o in parts)),
        "batched": {"mvis_per_s": nvis / (ms_b * 1e-3) / 1e6, "ms_per_step": ms_b, "form": "one CUDA graph"},
        "plain": {"mvis_per_s": nvis / (ms_p * 1e-3) / 1e6, "ms_per_step": ms_p, "form": "direct calls"},
        "ratio": ms_p / ms_b,
        "grid_rel_diff": rel(grid_b, grid_p),
        "vis_rel_diff": max(rel(d["vout_b"], d["vout_p"]) for _, d, _ in groups),
        "tuned_shapes": tuned,
        "steps": args.steps,
        "warmup": args.warmup,
    }
    cyc.close()
    for _, _, p in groups:
        p.close()
    return line


def main(argv=None):
    line = run(parse(argv))
    print(json.dumps(line), flush=True)
    return line


if __name__ == "__main__":
    main()
