"""Precision sweep on the config-3 generator: the full 100-station geometry
(a disk 100 km across, baselines to 97.6 km), 64 channels over 100-200 MHz,
subgrids of 32^2 and 64^2, planned with channel and time splitting
(datasets.plan_subgrids_split).

The sample (datasets.config3_sample) takes two baselines from every decile of
baseline length over all 4950 baselines, plus the longest, over a 512-step
window of the 8192-step observation, so that the FP64 oracle finishes in
seconds; uvw is computed for those baselines only.  For a seeded sample of
subgrids from every decile -- always including the longest baseline's -- the
gridder's subgrids and the degridder's visibilities of both variants are
compared with the FP64 oracle of the same gridder/degridder.  Relative RMS and
maximum error (max |got - want| over the RMS of want) are printed per decile as
one JSON line each, and the relative RMS is held to the 1e-5 tolerance overall
and in every decile.  This is where the reference's FP32 phase
(gridding/src/gridding_benchmark.cpp:77-81, :118-124) cancels worst.
"""
import json

import numpy as np
import pytest

import idg_gb300._lib as L
from gpu_helpers import degrid_gpu, grid_gpu, spec_for
from test_gpu_kernels import _oracle_with_ext

pytestmark = pytest.mark.gpu

TOL = 1e-5
PER_DECILE = 16


def _decile_errors(got, want, decile, nd=10):
    out = []
    for d in range(nd):
        sel = decile == d
        if not np.any(sel):
            continue
        g, w = got[sel], want[sel]
        scale = np.sqrt(np.mean(np.abs(w) ** 2))
        out.append({"decile": d, "rel_rms": float(np.linalg.norm(g - w) / np.linalg.norm(w)),
                    "max_err": float(np.abs(g - w).max() / scale)})
    return out


def _sample(oracle_mod, S):
    """Config-3 sample, a seeded sample of PER_DECILE subgrids per baseline
    decile (plus the longest baseline's first subgrids), random visibilities /
    subgrids and the FP64 oracle's outputs."""
    from idg_gb300 import datasets as D

    obs, bl_dec, edges, bl_len = D.config3_sample(S)
    spec = obs.spec
    md_all, ext_all = obs.metadata, obs.ext
    C = spec.nchannels
    sub_bl = md_all["time_offset"] // spec.ntimesteps
    dec_all = bl_dec[sub_bl]
    longest = np.where(sub_bl == int(np.argmax(bl_len)))[0]
    assert bl_len.max() >= 95e3 and bl_dec[np.argmax(bl_len)] == 9
    rng = np.random.default_rng(7 + S)
    pick = np.concatenate([rng.choice(np.where(dec_all == d)[0], min(PER_DECILE, int((dec_all == d).sum())),
                                      replace=False) for d in range(10)] + [longest[:4], longest[-4:]])
    pick = np.unique(pick)
    md, ext, dec = md_all[pick].copy(), ext_all[pick].copy(), dec_all[pick]
    N = md.shape[0]
    rows = obs.uvw.shape[0]
    vis = (rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64)
    sub_in = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    want_g, want_v = _oracle_with_ext(oracle_mod, spec.grid_size, S, spec.nstations, spec.image_size, obs.uvw,
                                      obs.wavenumbers, vis, obs.taper, obs.aterms, md, ext, sub_in)
    covered = np.zeros((rows, C), bool)
    vdec = np.full((rows, C), -1)
    for m, e, d in zip(md, ext, dec):
        r = slice(int(m["time_offset"]), int(m["time_offset"]) + int(m["nr_timesteps"]))
        covered[r, e["channel_begin"]:e["channel_end"]] = True
        vdec[r, e["channel_begin"]:e["channel_end"]] = d
    return spec, obs, md, ext, dec, edges, vis, sub_in, want_g, want_v, covered, vdec, float(bl_len.max()) / 1e3


@pytest.mark.parametrize("S", [32, 64])
def test_precision_sweep_by_baseline_decile(oracle_mod, idg, S):
    spec, obs, md, ext, dec, edges, vis, sub_in, want_g, want_v, covered, vdec, top_km = _sample(oracle_mod, S)
    N, C, rows = md.shape[0], spec.nchannels, obs.uvw.shape[0]
    sp = spec_for(spec.grid_size, S, C, spec.nstations, obs.aterms.shape[0], spec.image_size)
    for variant in (L.VARIANT_PLAIN, L.VARIANT_BATCHED):
        got_g = grid_gpu(sp, md, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, variant, ext=ext)
        got_v = degrid_gpu(sp, md, obs.uvw, obs.wavenumbers, sub_in, obs.taper, obs.aterms, rows, variant, ext=ext)
        gd = _decile_errors(got_g.reshape(N, -1), want_g.reshape(N, -1), dec)
        vd = _decile_errors(got_v[covered], want_v[covered], vdec[covered])
        overall_g = float(np.linalg.norm(got_g - want_g) / np.linalg.norm(want_g))
        overall_v = float(np.linalg.norm(got_v[covered] - want_v[covered]) / np.linalg.norm(want_v[covered]))
        for name, table, overall in (("grid", gd, overall_g), ("vis", vd, overall_v)):
            line = {"S": S, "variant": "batched" if variant == L.VARIANT_BATCHED else "plain", "output": name,
                    "subgrids": int(N), "overall_rel_rms": overall,
                    "worst_decile_rel_rms": max(t["rel_rms"] for t in table),
                    "top_decile_rel_rms": table[-1]["rel_rms"], "longest_baseline_km": round(top_km, 1),
                    "baseline_decile_edges_km": [round(float(x) / 1e3, 1) for x in edges], "deciles": table}
            print("[precision] " + json.dumps(line))
            assert overall <= TOL, line
            assert max(t["rel_rms"] for t in table) <= TOL, line
        assert np.all(got_v[~covered] == 0)


@pytest.mark.parametrize("S", [32, 64])
def test_channel_recurrence_precision_by_decile(oracle_mod, idg, S):
    """The batched gridder's channel-recurrence shapes on the precision sweep:
    64 channels whose float wavenumber steps take three values (chains break
    where a third one enters and every 16 channels), long baselines whose tiles
    fall back to per-channel sincos.  Same tolerance, per decile, as the
    per-channel form (whose error is printed beside it)."""
    from idg_gb300 import tuning

    spec, obs, md, ext, dec, edges, vis, sub_in, want_g, want_v, covered, vdec, _ = _sample(oracle_mod, S)
    N, C = md.shape[0], spec.nchannels
    steps = np.unique(np.diff(obs.wavenumbers))
    assert steps.size >= 3
    sp = spec_for(spec.grid_size, S, C, spec.nstations, obs.aterms.shape[0], spec.image_size)
    ng, _ = tuning.num_shapes()
    saved = tuning.get_shapes(S)
    try:
        for shape in [13] + list(range(15, ng)):
            tuning.set_shapes(S, shape, saved[1])
            got_g = grid_gpu(sp, md, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, L.VARIANT_BATCHED, ext=ext)
            gd = _decile_errors(got_g.reshape(N, -1), want_g.reshape(N, -1), dec)
            overall = float(np.linalg.norm(got_g - want_g) / np.linalg.norm(want_g))
            print("[precision] " + json.dumps({"S": S, "gridder_shape": shape, "overall_rel_rms": overall,
                                               "worst_decile_rel_rms": max(t["rel_rms"] for t in gd)}))
            assert overall <= TOL and max(t["rel_rms"] for t in gd) <= TOL, (shape, gd)
    finally:
        tuning.set_shapes(S, *saved)
