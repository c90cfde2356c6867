"""Batched uneven subgrids (config-4 generator, reduced): timesteps per subgrid
log-uniform in [16, 256], channel groups of 8/16/32/64 of 64 channels, subgrid
sizes 24, 32 and 48, an 8192^2 grid.

* Each size's gridder and degridder outputs, both variants, against the FP64
  oracle (relative RMS <= 1e-5).
* The whole job -- one plan per subgrid size (longest-first work lists, tuned
  launch shapes), all sharing one grid -- captured as one CUDA graph
  (idg_cycle_capture) and replayed: grid and predicted visibilities equal the
  direct gridding/degridding steps of the plain variant within 1e-5.
"""
import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from conftest import check_rel
from gpu_helpers import degrid_gpu, dev, grid_gpu, spec_for
from test_gpu_kernels import _oracle_with_ext

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _parts():
    from idg_gb300 import datasets as D

    parts = D.config4(n_subgrids=96, nstations=48, seed=41)
    rng = np.random.default_rng(42)
    out = []
    for o in parts:
        rows, C = o.uvw.shape[0], o.spec.nchannels
        vis = (rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64)
        out.append((o, vis))
    return out


def test_uneven_sizes_against_the_oracle(oracle_mod, idg):
    for o, vis in _parts():
        S, C, N = o.spec.subgrid_size, o.spec.nchannels, o.metadata.shape[0]
        rows = vis.shape[0]
        rng = np.random.default_rng(S)
        sub_in = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
        want_g, want_v = _oracle_with_ext(oracle_mod, o.spec.grid_size, S, o.spec.nstations, o.spec.image_size, o.uvw,
                                          o.wavenumbers, vis, o.taper, o.aterms, o.metadata, o.ext, sub_in)
        covered = np.zeros((rows, C), bool)
        for m, e in zip(o.metadata, o.ext):
            covered[m["time_offset"]:m["time_offset"] + m["nr_timesteps"], e["channel_begin"]:e["channel_end"]] = True
        sp = spec_for(o.spec.grid_size, S, C, o.spec.nstations, 1, o.spec.image_size)
        for variant in (L.VARIANT_PLAIN, L.VARIANT_BATCHED):
            got = grid_gpu(sp, o.metadata, o.uvw, o.wavenumbers, vis, o.taper, o.aterms, variant, ext=o.ext)
            check_rel(f"config-4 gridder S={S} v{variant}", got, want_g, TOL)
            vg = degrid_gpu(sp, o.metadata, o.uvw, o.wavenumbers, sub_in, o.taper, o.aterms, rows, variant, ext=o.ext)
            check_rel(f"config-4 degridder S={S} v{variant}", vg[covered], want_v[covered], TOL)


def test_mixed_size_job_as_one_graph(idg):
    from idg_gb300 import ops, tuning

    parts = _parts()
    G = parts[0][0].spec.grid_size
    grid_ref = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
    grid = torch.full_like(grid_ref, 3.0)
    plans, args, refs, dd = [], [], [], []
    for o, vis in parts:
        S, C, N = o.spec.subgrid_size, o.spec.nchannels, o.metadata.shape[0]
        sp = spec_for(G, S, C, o.spec.nstations, 1, o.spec.image_size)
        d = dict(md=dev(o.metadata), uvw=dev(o.uvw), k=dev(o.wavenumbers), vis=dev(vis), taper=dev(o.taper),
                 at=dev(o.aterms), ext=ops.ext_tensor(o.ext, "cuda"))
        sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
        vout = torch.zeros_like(d["vis"])
        tuning.autotune(sp, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, vout, ext=d["ext"], repeats=1,
                        store=False)
        ops.grid_visibilities(sp, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, grid_ref,
                              variant=L.VARIANT_PLAIN, ext=d["ext"])
        dd.append((sp, d, sub))
        plans.append(ops.Plan(sp, o.metadata, vis.shape[0], ext=o.ext, variant=L.VARIANT_BATCHED))
        args.append((d["uvw"], d["k"], d["vis"], d["taper"], d["at"], torch.zeros_like(d["vis"])))
    for sp, d, sub in dd:
        vref = torch.zeros_like(d["vis"])
        ops.degrid_visibilities(sp, d["md"], d["uvw"], d["k"], vref, d["taper"], d["at"], sub, grid_ref,
                                variant=L.VARIANT_PLAIN, ext=d["ext"])
        refs.append(vref)
    cyc = ops.Cycle(plans, args, grid)
    for _ in range(2):
        cyc.launch()
    torch.cuda.synchronize()
    check_rel("config-4 one-graph grid", grid.cpu().numpy(), grid_ref.cpu().numpy(), TOL)
    for (o, _), a, vref in zip(parts, args, refs):
        check_rel(f"config-4 one-graph vis S={o.spec.subgrid_size}", a[5].cpu().numpy(), vref.cpu().numpy(), TOL)
    for p in plans:
        assert p.status() == 0
    cyc.close()
    for p in plans:
        p.close()
