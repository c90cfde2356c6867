"""Parity of the CUDA kernels (through the C ABI) with the FP64 oracle.

Tolerance: relative RMS error <= 1e-5 against the FP64 oracle evaluated on
the same float inputs, for gridder and degridder outputs (the benchmark's
accuracy target); the subgrid FFT, adder and splitter are FP32 transforms of
FP32 data and are held to 2e-6.
"""
import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from conftest import check_rel, golden_cases, load_golden, rel_rms
from gpu_helpers import degrid_gpu, dev, grid_gpu, spec_for

pytestmark = pytest.mark.gpu

TOL = 1e-5
VARIANTS = [L.VARIANT_PLAIN, L.VARIANT_BATCHED]


def _config1_obs(**over):
    from idg_gb300 import datasets as D

    spec = D.config1()
    for k, v in over.items():
        setattr(spec, k, v)
    return spec, D.make_observation(spec)


def _vis(spec, seed=7):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((spec.n_rows, spec.nchannels, 4)) +
            1j * rng.standard_normal((spec.n_rows, spec.nchannels, 4))).astype(np.complex64)


@pytest.mark.parametrize("variant", VARIANTS)
def test_gridder_config1_vs_fp64(oracle_mod, idg, variant):
    spec, obs = _config1_obs()
    vis = _vis(spec)
    sp = spec_for(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, obs.aterms.shape[0],
                  spec.image_size)
    got = grid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, variant)
    prm = oracle_mod.params(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, spec.n_subgrids,
                            spec.image_size)
    want = oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, obs.metadata)
    check_rel(f"gridder config1 v{variant}", got, want, TOL)


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("refcpu", [False, True])
def test_degridder_config1_vs_fp64(oracle_mod, idg, variant, refcpu):
    spec, obs = _config1_obs(aterm_sigma=0.05)
    rng = np.random.default_rng(11)
    S = spec.subgrid_size
    sub = (rng.standard_normal((spec.n_subgrids, 4, S, S)) + 1j * rng.standard_normal((spec.n_subgrids, 4, S, S))).astype(np.complex64)
    flags = L.IDG_FLAG_DEGRID_ATERM_REFCPU if refcpu else 0
    sp = spec_for(spec.grid_size, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size, flags=flags)
    got = degrid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, spec.n_rows, variant)
    prm = oracle_mod.params(spec.grid_size, S, spec.nchannels, spec.nstations, spec.n_subgrids, spec.image_size)
    want = oracle_mod.degridder(prm, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, obs.metadata, spec.n_rows,
                                aterm_mode=oracle_mod.ATERM_REFCPU if refcpu else oracle_mod.ATERM_ADJOINT)
    check_rel(f"degridder config1 v{variant} refcpu={refcpu}", got, want, TOL)


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.rsplit("/", 1)[-1])
def test_reference_inputs_gridder_and_degridder(oracle_mod, idg, path):
    """The reference's own inputs and random plan (image_size 0.1): FP64 oracle within 1e-5,
    and the reference's FP32 CPU output within its own FP32 error (5e-4)."""
    d = load_golden(path)
    G, S, ns, C, nts, T = d["cfg"]
    nsg = d["metadata"].shape[0]
    sp = spec_for(G, S, C, ns, nts, 0.1, flags=L.IDG_FLAG_DEGRID_ATERM_REFCPU)
    prm = oracle_mod.params(G, S, C, ns, nsg, 0.1)
    for variant in VARIANTS:
        got = grid_gpu(sp, d["metadata"], d["uvw"], d["wavenumbers"], d["vis"], d["spheroidal"], d["aterms"], variant)
        want = oracle_mod.gridder(prm, d["uvw"], d["wavenumbers"], d["vis"], d["spheroidal"], d["aterms"], d["metadata"])
        check_rel(f"gridder reference-inputs v{variant}", got, want, TOL)
        assert rel_rms(d["gridder_out"], got) < 5e-4
        vg = degrid_gpu(sp, d["metadata"], d["uvw"], d["wavenumbers"], d["degridder_in"], d["spheroidal"],
                        d["aterms"], d["vis"].shape[0], variant)
        vw = oracle_mod.degridder(prm, d["uvw"], d["wavenumbers"], d["degridder_in"], d["spheroidal"], d["aterms"],
                                  d["metadata"], d["vis"].shape[0], aterm_mode=oracle_mod.ATERM_REFCPU)
        check_rel(f"degridder reference-inputs v{variant}", vg, vw, TOL)
        assert rel_rms(d["degridder_out"], vg) < 5e-4


def test_config2_sample_vs_fp64(oracle_mod, idg):
    """48 subgrids of the full config-2 plan (including the longest baselines)."""
    from idg_gb300 import datasets as D

    spec = D.config2()
    obs = D.make_observation(spec)
    bl_len = np.linalg.norm(obs.uvw[:: spec.ntimesteps, :2], axis=1)
    order = np.argsort(bl_len)
    pick_bl = np.concatenate([order[:8], order[len(order) // 2: len(order) // 2 + 8], order[-8:]])
    subs = np.concatenate([b * spec.subgrids_per_baseline + np.array([0, spec.subgrids_per_baseline - 1]) for b in pick_bl])
    md = obs.metadata[subs].copy()
    # compact the rows these subgrids use
    rows = np.concatenate([np.arange(m["time_offset"], m["time_offset"] + m["nr_timesteps"]) for m in md])
    uvw = obs.uvw[rows]
    md["time_offset"] = np.arange(len(md)) * spec.timesteps_per_subgrid
    rng = np.random.default_rng(5)
    vis = (rng.standard_normal((len(rows), spec.nchannels, 4)) + 1j * rng.standard_normal((len(rows), spec.nchannels, 4))).astype(np.complex64)
    S = spec.subgrid_size
    sp = spec_for(spec.grid_size, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    prm = oracle_mod.params(spec.grid_size, S, spec.nchannels, spec.nstations, len(md), spec.image_size)
    want = oracle_mod.gridder(prm, uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, md)
    for variant in VARIANTS:
        got = grid_gpu(sp, md, uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, variant)
        check_rel(f"gridder config2-sample v{variant}", got, want, TOL)
    sub = (rng.standard_normal((len(md), 4, S, S)) + 1j * rng.standard_normal((len(md), 4, S, S))).astype(np.complex64)
    vwant = oracle_mod.degridder(prm, uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, md, len(rows))
    for variant in VARIANTS:
        vgot = degrid_gpu(sp, md, uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, len(rows), variant)
        check_rel(f"degridder config2-sample v{variant}", vgot, vwant, TOL)


@pytest.mark.parametrize("S", [8, 16, 24, 32, 48, 64])
def test_subgrid_fft_vs_dft(oracle_mod, idg, S):
    from idg_gb300 import ops

    rng = np.random.default_rng(S)
    N = 5
    P = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    taper = rng.random((S, S)).astype(np.float32)
    sp = spec_for(1024, S, 1, 2, 1, 0.05)
    for direction in (1, -1):
        for tp in (None, taper):
            x = dev(P)
            ops.subgrid_fft(sp, x, direction, dev(tp) if tp is not None else None)
            torch.cuda.synchronize()
            want = oracle_mod.subgrid_dft(P, direction, tp)
            assert rel_rms(x.cpu().numpy(), want) <= 2e-6, (direction, tp is not None)
    x = dev(P)
    ops.subgrid_fft(sp, x, 1)
    ops.subgrid_fft(sp, x, -1)
    torch.cuda.synchronize()
    assert rel_rms(x.cpu().numpy() / (S * S), P) <= 2e-6


def test_adder_splitter_vs_oracle(oracle_mod, idg):
    """Adder and splitter with w-planes, negative-w entries (mirrored, conjugated)
    and entries outside the planes or partly outside the grid."""
    from idg_gb300 import ops

    S, G, W = 16, 96, 2
    rng = np.random.default_rng(2)
    N = 40
    md = np.zeros(N, L.METADATA_DTYPE)
    md["x"] = rng.integers(-S + 2, G - 2, N)
    md["y"] = rng.integers(-S + 2, G - 2, N)
    md["z"] = rng.integers(-W, W, N)  # negative z: Hermitian mirror into plane -z-1
    md["z"][0] = 5  # outside the w-planes: skipped by the adder, zeros from the splitter
    md["z"][1] = -W - 1
    assert (md["z"] < 0).sum() >= 8
    sub = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    sp = spec_for(G, S, 1, 2, 1, 0.05, W=W)
    grid = torch.zeros((W, 4, G, G), dtype=torch.complex64, device="cuda")
    ops.adder(sp, dev(md), dev(sub), grid)
    torch.cuda.synchronize()
    want = oracle_mod.adder(sub, md, G, W)
    assert rel_rms(grid.cpu().numpy(), want) <= 2e-6
    g = (rng.standard_normal((W, 4, G, G)) + 1j * rng.standard_normal((W, 4, G, G))).astype(np.complex64)
    out = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    ops.splitter(sp, dev(md), dev(g), out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle_mod.splitter(g, md, S).astype(np.complex64))


@pytest.mark.parametrize("S", [8, 24, 32, 64])
def test_split_fft_pass_equals_splitter_then_fft(idg, S):
    """The degridding step reads the grid and runs the backward subgrid FFT in
    one pass: its subgrids equal the splitter followed by the backward FFT bit
    for bit, with w-planes, mirrored negative-w entries, entries outside the
    planes and footprints partly or wholly outside the grid."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config1()
    spec.subgrid_size = S
    obs = D.make_observation(spec)
    G, W, N = 160, 2, spec.n_subgrids
    rng = np.random.default_rng(S)
    md = obs.metadata.copy()
    md["x"] = rng.integers(-S + 2, G - 2, N)
    md["y"] = rng.integers(-S + 2, G - 2, N)
    md["z"] = rng.integers(-W, W, N)
    md["x"][:4] = [-S, G, G - S // 2 - 1, -S // 2 + 1]  # wholly outside / straddling the edges
    md["z"][4], md["z"][5] = W, -W - 1                   # outside the planes: zeros
    assert (md["z"] < 0).sum() >= 4
    sp = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size, W=W)
    g = dev((rng.standard_normal((W, 4, G, G)) + 1j * rng.standard_normal((W, 4, G, G))).astype(np.complex64))
    d = {k: dev(v) for k, v in dict(md=md, uvw=obs.uvw, k=obs.wavenumbers, taper=obs.taper, at=obs.aterms).items()}
    want = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    ops.splitter(sp, d["md"], g, want)
    ops.subgrid_fft(sp, want, -1, d["taper"])
    got = torch.empty_like(want)
    vis = torch.zeros((obs.uvw.shape[0], spec.nchannels, 4), dtype=torch.complex64, device="cuda")
    ops.degrid_visibilities(sp, d["md"], d["uvw"], d["k"], vis, d["taper"], d["at"], got, g)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), want.cpu().numpy())


def test_bad_plan_entry_is_flagged_not_faulted(idg):
    from idg_gb300 import ops

    spec, obs = _config1_obs()
    vis = _vis(spec)
    md = obs.metadata.copy()
    md["time_offset"][3] = spec.n_rows  # rows past the end
    md["station2"][5] = 999             # station out of range
    sp = spec_for(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, 1, spec.image_size)
    ops.device_status(clear=True)
    got = grid_gpu(sp, md, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms)
    assert ops.device_status(clear=True) & 1
    assert np.all(got[3] == 0) and np.all(got[5] == 0)
    assert np.any(got[4] != 0)
    assert ops.device_status(clear=True) == 0


def _oracle_with_ext(oracle_mod, G, S, ns, image_size, uvw, k, vis, taper, aterms, md, ext, sub_in=None, w_step=0.0):
    """FP64 oracle for plans whose subgrids cover channel ranges [c0, c1): one oracle
    call per distinct range on the sliced channel axis."""
    N, C = md.shape[0], k.shape[0]
    grid_out = np.zeros((N, 4, S, S), np.complex128)
    vis_out = np.zeros((vis.shape[0], C, 4), np.complex128)
    for c0, c1 in sorted(set(zip(ext["channel_begin"].tolist(), ext["channel_end"].tolist()))):
        sel = np.where((ext["channel_begin"] == c0) & (ext["channel_end"] == c1))[0]
        if c1 <= c0:
            continue
        prm = oracle_mod.params(G, S, c1 - c0, ns, len(sel), image_size, w_step)
        kk = np.ascontiguousarray(k[c0:c1])
        vv = np.ascontiguousarray(vis[:, c0:c1])
        mds = np.ascontiguousarray(md[sel])
        # the oracle reads rows relative to the first entry's baseline_offset (all zero here)
        grid_out[sel] = oracle_mod.gridder(prm, uvw, kk, vv, taper, aterms, mds)
        if sub_in is not None:
            part = oracle_mod.degridder(prm, uvw, kk, np.ascontiguousarray(sub_in[sel]), taper, aterms, mds,
                                        vis.shape[0])
            for m in mds:
                r0, r1 = m["time_offset"], m["time_offset"] + m["nr_timesteps"]
                vis_out[r0:r1, c0:c1] = part[r0:r1]
    return grid_out, vis_out


@pytest.mark.parametrize("S", [24, 48, 64])
def test_uneven_plan_channel_groups(oracle_mod, idg, S):
    """Uneven subgrids in one launch: random timesteps per subgrid, channel ranges from
    the sidecar, non-overlapping rows; subgrid sizes needing 1, 3 and 4 pixel passes."""
    from idg_gb300 import datasets as D

    rng = np.random.default_rng(100 + S)
    G, C, ns = 2048, 24, 6
    image_size = 0.04
    spec = D.ObservationSpec(nstations=ns, disk_radius_m=2500.0, ntimesteps=160, timesteps_per_subgrid=160,
                             nchannels=C, f_start=140e6, f_end=170e6, subgrid_size=S, grid_size=G,
                             image_size=image_size, aterm_sigma=0.05, seed=S)
    obs = D.make_observation(spec)
    N = 20
    T = rng.integers(5, 41, N)
    md = np.zeros(N, L.METADATA_DTYPE)
    md["time_offset"] = np.concatenate([[0], np.cumsum(T)[:-1]])
    md["nr_timesteps"] = T
    md["station1"] = rng.integers(0, ns - 1, N)
    md["station2"] = md["station1"] + 1
    md["x"] = rng.integers(0, G - S, N)
    md["y"] = rng.integers(0, G - S, N)
    lens = rng.choice([3, 8, 16, 24], N)
    c0 = np.array([rng.integers(0, C - L_ + 1) for L_ in lens])
    ext = np.zeros(N, L.SUBGRID_EXT_DTYPE)
    ext["channel_begin"] = c0
    ext["channel_end"] = c0 + lens
    rows = int(T.sum())
    uvw = np.ascontiguousarray(obs.uvw[:rows])
    vis = (rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64)
    sub_in = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    want_g, want_v = _oracle_with_ext(oracle_mod, G, S, ns, image_size, uvw, obs.wavenumbers, vis, obs.taper,
                                      obs.aterms, md, ext, sub_in)
    sp = spec_for(G, S, C, ns, obs.aterms.shape[0], image_size)
    covered = np.zeros((rows, C), bool)
    for m, e in zip(md, ext):
        covered[m["time_offset"]:m["time_offset"] + m["nr_timesteps"], e["channel_begin"]:e["channel_end"]] = True
    for variant in VARIANTS:
        got = grid_gpu(sp, md, uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, variant, ext=ext)
        check_rel(f"gridder uneven S={S} v{variant}", got, want_g, TOL)
        vg = degrid_gpu(sp, md, uvw, obs.wavenumbers, sub_in, obs.taper, obs.aterms, rows, variant, ext=ext)
        check_rel(f"degridder uneven S={S} v{variant}", vg[covered], want_v[covered], TOL)
        assert np.all(vg[~covered] == 0)


def test_large_phase_path(oracle_mod, idg):
    """Subgrids whose per-channel phase exceeds the unreduced-sincos bound take the
    reduced path in the batched kernels; both variants stay within tolerance."""
    from idg_gb300 import datasets as D

    spec = D.ObservationSpec(nstations=5, disk_radius_m=10000.0, ntimesteps=32, timesteps_per_subgrid=32,
                             nchannels=16, f_start=150e6, f_end=170e6, subgrid_size=64, grid_size=4096,
                             image_size=0.05, seed=9)
    obs = D.make_observation(spec)
    vis = _vis(spec, seed=3)
    sp = spec_for(spec.grid_size, 64, 16, 5, 1, spec.image_size)
    prm = oracle_mod.params(spec.grid_size, 64, 16, 5, spec.n_subgrids, spec.image_size)
    want = oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, obs.metadata)
    for variant in VARIANTS:
        got = grid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, variant)
        check_rel(f"gridder large-phase v{variant}", got, want, TOL)
    rng = np.random.default_rng(4)
    sub = (rng.standard_normal((spec.n_subgrids, 4, 64, 64)) + 1j * rng.standard_normal((spec.n_subgrids, 4, 64, 64))).astype(np.complex64)
    vwant = oracle_mod.degridder(prm, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, obs.metadata, spec.n_rows)
    for variant in VARIANTS:
        vgot = degrid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, spec.n_rows, variant)
        check_rel(f"degridder large-phase v{variant}", vgot, vwant, TOL)
    # every batched shape on the reduced path
    from idg_gb300 import tuning

    ng, nd = tuning.num_shapes()
    saved = tuning.get_shapes(64)
    for sh in range(max(ng, nd)):
        tuning.set_shapes(64, min(sh, ng - 1), min(sh, nd - 1))
        if sh < ng:
            got = grid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, L.VARIANT_BATCHED)
            check_rel(f"gridder large-phase shape {sh}", got, want, TOL)
        if sh < nd:
            vgot = degrid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, spec.n_rows,
                              L.VARIANT_BATCHED)
            check_rel(f"degridder large-phase shape {sh}", vgot, vwant, TOL)
    tuning.set_shapes(64, *saved)


def test_every_batched_shape_and_the_autotuner(oracle_mod, idg):
    """Each compiled launch shape of the batched kernels gives the same parity; the
    autotuner times them all and leaves the fastest selected."""
    from idg_gb300 import tuning

    spec, obs = _config1_obs(aterm_sigma=0.05)
    vis = _vis(spec, seed=12)
    S = spec.subgrid_size
    sp = spec_for(spec.grid_size, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    prm = oracle_mod.params(spec.grid_size, S, spec.nchannels, spec.nstations, spec.n_subgrids, spec.image_size)
    want = oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, obs.metadata)
    rng = np.random.default_rng(13)
    sub = (rng.standard_normal((spec.n_subgrids, 4, S, S)) + 1j * rng.standard_normal((spec.n_subgrids, 4, S, S))).astype(np.complex64)
    vwant = oracle_mod.degridder(prm, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, obs.metadata, spec.n_rows)
    ng, nd = tuning.num_shapes()
    assert ng >= 2 and nd >= 2
    saved = tuning.get_shapes(S)
    for sh in range(max(ng, nd)):
        tuning.set_shapes(S, min(sh, ng - 1), min(sh, nd - 1))
        got = grid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, L.VARIANT_BATCHED)
        check_rel(f"gridder shape {min(sh, ng - 1)}", got, want, TOL)
        vg = degrid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, sub, obs.taper, obs.aterms, spec.n_rows,
                        L.VARIANT_BATCHED)
        check_rel(f"degridder shape {min(sh, nd - 1)}", vg, vwant, TOL)
    # autotuner on device data
    d = {k: dev(v) for k, v in dict(md=obs.metadata, uvw=obs.uvw, k=obs.wavenumbers, vis=vis, taper=obs.taper,
                                    at=obs.aterms).items()}
    out_sub = torch.empty((spec.n_subgrids, 4, S, S), dtype=torch.complex64, device="cuda")
    out_vis = torch.empty_like(d["vis"])
    res = tuning.autotune(sp, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], out_sub, out_vis, repeats=1,
                          store=False)
    assert len(res["gridder_ms"]) == ng and all(t > 0 for t in res["gridder_ms"])
    assert tuning.get_shapes(S) == (res["gridder"], res["degridder"])
    # the fastest shape, or the one in use before when within 1 % of it
    assert res["gridder_ms"][res["gridder"]] <= 1.01 * min(res["gridder_ms"]) + 1e-9
    assert res["degridder_ms"][res["degridder"]] <= 1.01 * min(res["degridder_ms"]) + 1e-9
    tuning.set_shapes(S, *saved)


@pytest.mark.parametrize("S", [8, 16, 20, 24, 36, 48, 64])
def test_every_batched_shape_at_other_subgrid_sizes(oracle_mod, idg, S):
    """Every launch shape of both batched kernels (pixel-pair and channel-pair
    degridders included) on an uneven plan with subgrid sizes that need partial
    pixel passes and channel ranges that are not multiples of the channel group.
    S = 20 and 36 have S/2 not a multiple of 4: the column-form degridder's
    lanes then change column at different steps (divergent P updates)."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops, tuning

    rng = np.random.default_rng(200 + S)
    G, C, ns = 2048, 20, 5
    image_size = 0.04
    spec = D.ObservationSpec(nstations=ns, disk_radius_m=2500.0, ntimesteps=120, timesteps_per_subgrid=120,
                             nchannels=C, f_start=140e6, f_end=170e6, subgrid_size=S, grid_size=G,
                             image_size=image_size, aterm_sigma=0.05, seed=S + 1)
    obs = D.make_observation(spec)
    N = 8
    T = rng.integers(4, 16, N)
    md = np.zeros(N, L.METADATA_DTYPE)
    md["time_offset"] = np.concatenate([[0], np.cumsum(T)[:-1]])
    md["nr_timesteps"] = T
    md["station1"] = rng.integers(0, ns - 1, N)
    md["station2"] = md["station1"] + 1
    md["x"] = rng.integers(0, G - S, N)
    md["y"] = rng.integers(0, G - S, N)
    lens = rng.choice([3, 8, 13, 20], N)
    c0 = np.array([rng.integers(0, C - L_ + 1) for L_ in lens])
    ext = np.zeros(N, L.SUBGRID_EXT_DTYPE)
    ext["channel_begin"] = c0
    ext["channel_end"] = c0 + lens
    rows = int(T.sum())
    uvw = np.ascontiguousarray(obs.uvw[:rows])
    vis = (rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64)
    sub_in = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    want_g, want_v = _oracle_with_ext(oracle_mod, G, S, ns, image_size, uvw, obs.wavenumbers, vis, obs.taper,
                                      obs.aterms, md, ext, sub_in)
    covered = np.zeros((rows, C), bool)
    for m, e in zip(md, ext):
        covered[m["time_offset"]:m["time_offset"] + m["nr_timesteps"], e["channel_begin"]:e["channel_end"]] = True
    sp = spec_for(G, S, C, ns, obs.aterms.shape[0], image_size)
    ng, nd = tuning.num_shapes()
    saved = tuning.get_shapes(S)
    for sh in range(max(ng, nd)):
        g_sh, d_sh = min(sh, ng - 1), min(sh, nd - 1)
        tuning.set_shapes(S, g_sh, d_sh)
        if sh < ng:
            got = grid_gpu(sp, md, uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, L.VARIANT_BATCHED, ext=ext)
            check_rel(f"gridder S={S} shape {g_sh}", got, want_g, TOL)
        vg = degrid_gpu(sp, md, uvw, obs.wavenumbers, sub_in, obs.taper, obs.aterms, rows, L.VARIANT_BATCHED, ext=ext)
        check_rel(f"degridder S={S} shape {d_sh}", vg[covered], want_v[covered], TOL)
        assert np.all(vg[~covered] == 0)
    assert ops.device_status(clear=True) == 0
    tuning.set_shapes(S, *saved)


def test_plan_steps_and_graph_cycle_match_direct_calls(oracle_mod, idg):
    """A plan's grid/degrid steps and its captured CUDA-graph cycle reproduce the
    direct entry points; an uneven plan (longest-first work list) stays within tolerance."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config1()
    spec.aterm_sigma = 0.05
    obs = D.make_observation(spec)
    vis = _vis(spec, seed=31)
    S, G = spec.subgrid_size, spec.grid_size
    gs = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    d = {k: dev(v) for k, v in dict(md=obs.metadata, uvw=obs.uvw, k=obs.wavenumbers, vis=vis, taper=obs.taper,
                                    at=obs.aterms).items()}
    N = spec.n_subgrids
    # direct calls
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    g_ref = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
    ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, g_ref)
    v_ref = torch.zeros_like(d["vis"])
    ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], v_ref, d["taper"], d["at"], sub, g_ref)
    torch.cuda.synchronize()
    # oracle of the gridding step: gridder (no taper) -> DFT (+1, taper) -> adder
    prm = oracle_mod.params(G, S, spec.nchannels, spec.nstations, N, spec.image_size)
    ones = np.ones((S, S), np.float32)
    want_grid = oracle_mod.adder(oracle_mod.subgrid_dft(
        oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, vis, ones, obs.aterms, obs.metadata), +1, obs.taper),
        obs.metadata, G)
    check_rel("grid step vs oracle", g_ref.cpu().numpy(), want_grid, TOL)
    for variant in VARIANTS:
        plan = ops.Plan(gs, obs.metadata, spec.n_rows, variant=variant)
        g = torch.zeros_like(g_ref)
        plan.grid(d["uvw"], d["k"], d["vis"], d["taper"], d["at"], g)
        v = torch.zeros_like(d["vis"])
        plan.degrid(d["uvw"], d["k"], v, d["taper"], d["at"], g)
        torch.cuda.synchronize()
        check_rel(f"plan grid v{variant}", g.cpu().numpy(), g_ref.cpu().numpy(), TOL)
        check_rel(f"plan degrid v{variant}", v.cpu().numpy(), v_ref.cpu().numpy(), TOL)
        g2 = torch.full_like(g_ref, 7.0)
        v2 = torch.zeros_like(d["vis"])
        plan.capture_cycle(d["uvw"], d["k"], d["vis"], d["taper"], d["at"], g2, v2)
        for _ in range(2):
            plan.launch_cycle()
        torch.cuda.synchronize()
        check_rel(f"graph cycle grid v{variant}", g2.cpu().numpy(), g_ref.cpu().numpy(), TOL)
        check_rel(f"graph cycle vis v{variant}", v2.cpu().numpy(), v_ref.cpu().numpy(), TOL)
        assert plan.status() == 0
        plan.close()


def test_host_buffer_cycle_auto_chunks(idg):
    """IDG_CHUNKS_AUTO on 8192 config-2 subgrids: chunks growing through the
    gridding phase and shrinking through the degridding phase (several of
    each), uvw rows travelling with their chunk; same grid and visibilities as
    the device-resident steps."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config2()
    obs = D.truncate_observation(D.make_observation(spec), 8192)
    spec = obs.spec
    S, G, N = spec.subgrid_size, spec.grid_size, spec.n_subgrids
    gs = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    vis_d = D.visibilities(spec, device="cuda", seed=41)
    d = {k: dev(v) for k, v in dict(md=obs.metadata, uvw=obs.uvw, k=obs.wavenumbers, taper=obs.taper,
                                    at=obs.aterms).items()}
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    g_ref = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
    ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], vis_d, d["taper"], d["at"], sub, g_ref)
    v_ref = torch.zeros_like(vis_d)
    ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], v_ref, d["taper"], d["at"], sub, g_ref)
    torch.cuda.synchronize()
    vis_h = vis_d.cpu().numpy()
    out_h = np.zeros_like(vis_h)
    grid_h = np.zeros((1, 4, G, G), np.complex64)
    for mode in (L.CHUNKS_AUTO, L.CHUNKS_ADAPTIVE, L.CHUNKS_ADAPTIVE):
        out_h[...] = 0
        grid_h[...] = 0
        t = ops.imaging_cycle(gs, obs.metadata, obs.uvw, obs.wavenumbers, vis_h, obs.taper,
                              np.ascontiguousarray(obs.aterms), out_h, grid_out=grid_h, chunk_subgrids=mode)
        print(f"[cycle] chunks {mode}: {t['grid_chunks']} gridding, {t['degrid_chunks']} degridding, "
              f"ratio {t['chunk_ratio']:.3f}, gridding waited {t['gridding_wait_ms']:.2f} of {t['gridding_ms']:.2f} ms")
        assert t["grid_chunks"] > 1 and t["degrid_chunks"] > 1
        assert 1.1 <= t["chunk_ratio"] <= 1.6 and 0 <= t["gridding_wait_ms"] <= t["gridding_ms"]
        assert t["h2d_bytes"] >= vis_h.nbytes + obs.uvw.nbytes
        check_rel(f"host cycle chunks {mode} grid", grid_h, g_ref.cpu().numpy(), TOL)
        check_rel(f"host cycle chunks {mode} vis", out_h, v_ref.cpu().numpy(), TOL)
    ops.release_buffers()


def test_imaging_cycles_of_different_sizes(idg):
    """One idg_imaging_cycles call over config-1 observations of 14, 28 and 7
    subgrids (rows 896, 1792, 448): device buffers sized by the largest cycle,
    the plan and uvw of alternate cycles in alternate buffers; each cycle
    equals the device-resident steps on its own inputs, in chunks of 5."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config1()
    spec.aterm_sigma = 0.05
    full = D.make_observation(spec)
    S, G = spec.subgrid_size, spec.grid_size
    gs = spec_for(G, S, spec.nchannels, spec.nstations, full.aterms.shape[0], spec.image_size)
    at = np.ascontiguousarray(full.aterms)
    cycles, refs = [], []
    for n, seed in ((14, 71), (28, 72), (7, 73)):
        obs = D.truncate_observation(full, n)
        vis = _vis(obs.spec, seed=seed)
        assert obs.metadata.shape[0] == n and vis.shape[0] == obs.uvw.shape[0]
        d = {k: dev(x) for k, x in dict(md=obs.metadata, uvw=obs.uvw, k=obs.wavenumbers, vis=vis, taper=obs.taper,
                                        at=obs.aterms).items()}
        sub = torch.empty((n, 4, S, S), dtype=torch.complex64, device="cuda")
        g = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
        ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, g)
        vo = torch.zeros_like(d["vis"])
        ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], vo, d["taper"], d["at"], sub, g)
        torch.cuda.synchronize()
        refs.append((g.cpu().numpy(), vo.cpu().numpy()))
        cycles.append((obs.metadata, obs.uvw, vis, np.full(vis.shape, np.nan + 1j * np.nan, np.complex64),
                       np.zeros((1, 4, G, G), np.complex64)))
    try:
        ts = ops.imaging_cycles(gs, cycles, full.wavenumbers, full.taper, at, chunk_subgrids=5)
        for i, ((g_ref, v_ref), c) in enumerate(zip(refs, cycles)):
            check_rel(f"cycles of sizes [{i}] grid", c[4], g_ref, TOL)
            check_rel(f"cycles of sizes [{i}] vis", c[3], v_ref, TOL)
            assert ts[i]["h2d_vis_bytes"] == c[2].nbytes and ts[i]["d2h_vis_bytes"] == c[2].nbytes
            assert ts[i]["h2d_vis_ms"] > 0 and ts[i]["h2d_span_ms"] >= ts[i]["h2d_vis_ms"] - 0.01
    finally:
        ops.release_buffers()


@pytest.mark.parametrize("mode", [L.CHUNKS_AUTO, L.CHUNKS_ADAPTIVE])
def test_imaging_cycles_config2_chunked(idg, mode):
    """Three cycles of one idg_imaging_cycles call on 8192 config-2 subgrids,
    inputs A, B, A with outputs of their own: each chunk of a cycle's
    visibilities is copied in once the previous cycle's gridding chunks that
    read those rows have ended, while that cycle still grids its later chunks.
    Every cycle's grid and visibilities equal the device-resident steps on its
    own inputs (a copy that overwrote rows still to be gridded would mix B into
    A's grid).  Chunks: ten for the first gridding and the last degridding,
    four elsewhere (fewer where chunks under 1024 subgrids merge)."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config2()
    obs = D.truncate_observation(D.make_observation(spec), 8192)
    spec = obs.spec
    S, G, N = spec.subgrid_size, spec.grid_size, spec.n_subgrids
    gs = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    d = {k: dev(v) for k, v in dict(md=obs.metadata, uvw=obs.uvw, k=obs.wavenumbers, taper=obs.taper,
                                    at=obs.aterms).items()}
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    vis_h, refs = [], []
    for seed in (61, 62):
        vis_d = D.visibilities(spec, device="cuda", seed=seed)
        g = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
        ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], vis_d, d["taper"], d["at"], sub, g)
        vo = torch.zeros_like(vis_d)
        ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], vo, d["taper"], d["at"], sub, g)
        torch.cuda.synchronize()
        vis_h.append(vis_d.cpu().numpy())
        refs.append((g.cpu().numpy(), vo.cpu().numpy()))
        del vis_d, vo, g
    order = [0, 1, 0]
    outs = [np.zeros_like(vis_h[0]) for _ in order]
    grids = [np.zeros((1, 4, G, G), np.complex64) for _ in order]
    try:
        ts = ops.imaging_cycles(gs, [(obs.metadata, obs.uvw, vis_h[o], outs[i], grids[i]) for i, o in enumerate(order)],
                                obs.wavenumbers, obs.taper, np.ascontiguousarray(obs.aterms), chunk_subgrids=mode)
        for i, o in enumerate(order):
            t = ts[i]
            print(f"[cycles] {i}: {t['grid_chunks']} + {t['degrid_chunks']} chunks, gridding waited "
                  f"{t['gridding_wait_ms']:.2f} of {t['gridding_ms']:.2f} ms, ends at {t['end_ms']:.1f} ms")
            check_rel(f"cycles config2 [{i}] grid", grids[i], refs[o][0], TOL)
            check_rel(f"cycles config2 [{i}] vis", outs[i], refs[o][1], TOL)
            assert t["h2d_vis_bytes"] == vis_h[0].nbytes and t["d2h_vis_bytes"] == vis_h[0].nbytes
        assert ts[0]["grid_chunks"] > ts[1]["grid_chunks"] >= 2 and ts[2]["degrid_chunks"] > ts[1]["degrid_chunks"] >= 2
    finally:
        ops.release_buffers()


@pytest.mark.parametrize("chunk", [0, 5, -1, -2])
@pytest.mark.parametrize("locked", [False, True])
def test_host_buffer_cycle_matches_device_steps(idg, chunk, locked):
    """idg_imaging_cycle on host buffers (pageable numpy arrays, or page-locked
    huge-page arrays from idg_gb300.hostmem), in one chunk or in chunks of 5
    subgrids with the copies overlapping the kernels, gives the grid and the
    visibilities of the device-resident gridding and degridding steps."""
    from idg_gb300 import datasets as D
    from idg_gb300 import hostmem, ops

    spec = D.config1()
    spec.aterm_sigma = 0.05
    obs = D.make_observation(spec)
    vis = _vis(spec, seed=37)
    S, G, N = spec.subgrid_size, spec.grid_size, spec.n_subgrids
    gs = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    d = {k: dev(v) for k, v in dict(md=obs.metadata, uvw=obs.uvw, k=obs.wavenumbers, vis=vis, taper=obs.taper,
                                    at=obs.aterms).items()}
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    g_ref = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
    ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, g_ref)
    v_ref = torch.zeros_like(d["vis"])
    ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], v_ref, d["taper"], d["at"], sub, g_ref)
    torch.cuda.synchronize()

    if locked:
        host = [hostmem.pinned_copy(a) for a in (obs.metadata, obs.uvw, vis, obs.aterms)]
        md_h, uvw_h, vis_h, at_h = host
        out_h = hostmem.pinned_empty(vis.shape, np.complex64)
        grid_h = hostmem.pinned_empty((1, 4, G, G), np.complex64)
        host += [out_h, grid_h]
    else:
        host = []
        md_h, uvw_h, vis_h, at_h = obs.metadata, obs.uvw, vis, obs.aterms
        out_h = np.zeros(vis.shape, np.complex64)
        grid_h = np.zeros((1, 4, G, G), np.complex64)
    try:
        for _ in range(2):  # the second call reuses the cycle's device buffers
            t = ops.imaging_cycle(gs, md_h, uvw_h, obs.wavenumbers, vis_h, obs.taper, at_h, out_h, grid_out=grid_h,
                                  chunk_subgrids=chunk)
        check_rel(f"host cycle grid chunk={chunk} locked={locked}", grid_h, g_ref.cpu().numpy(), TOL)
        check_rel(f"host cycle vis chunk={chunk} locked={locked}", out_h, v_ref.cpu().numpy(), TOL)
        assert t["h2d_bytes"] >= vis.nbytes and t["d2h_bytes"] >= vis.nbytes + grid_h.nbytes
        assert t["total_ms"] > 0 and t["gridding_ms"] > 0 and t["degridding_ms"] > 0
    finally:
        ops.release_buffers()
        for a in host:
            hostmem.release(a)


@pytest.mark.parametrize("chunk", [L.CHUNKS_AUTO, 5])
def test_host_buffer_cycle_zeroes_rows_no_entry_names(idg, chunk):
    """A plan that names only some of the rows (every third config-1 subgrid
    dropped, and the first and the last): idg_imaging_cycle writes the
    degridded rows and zeros exactly in the rows no entry names, whatever the
    output buffer held before -- in one chunk, and in chunks of 5 subgrids,
    where unnamed rows lie before the first chunk, between two chunks' rows
    and after the last chunk."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config1()
    obs = D.make_observation(spec)
    vis = _vis(spec, seed=43)
    keep = np.arange(spec.n_subgrids) % 3 != 1
    keep[0] = keep[-1] = False
    md = np.ascontiguousarray(obs.metadata[keep])
    S, G, N = spec.subgrid_size, spec.grid_size, int(keep.sum())
    gs = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    d = {k: dev(v) for k, v in dict(md=md, uvw=obs.uvw, k=obs.wavenumbers, vis=vis, taper=obs.taper,
                                    at=obs.aterms).items()}
    sub = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    g_ref = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
    ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, g_ref)
    v_ref = torch.zeros_like(d["vis"])
    ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], v_ref, d["taper"], d["at"], sub, g_ref)
    torch.cuda.synchronize()
    named = np.zeros(vis.shape[0], bool)
    b0 = int(md["baseline_offset"][0])
    for m in md:
        r = int(m["baseline_offset"]) - b0 + int(m["time_offset"])
        named[r:r + int(m["nr_timesteps"])] = True
    assert named.any() and not named.all()
    out_h = np.full(vis.shape, np.nan + 1j * np.nan, np.complex64)
    try:
        t = ops.imaging_cycle(gs, md, obs.uvw, obs.wavenumbers, vis, obs.taper, np.ascontiguousarray(obs.aterms),
                              out_h, chunk_subgrids=chunk)
        assert np.all(out_h[~named] == 0)
        check_rel(f"host cycle vis, rows named, chunk={chunk}", out_h[named], v_ref.cpu().numpy()[named], TOL)
        assert t["total_ms"] > 0 and t["end_ms"] == t["total_ms"]
        assert t["d2h_vis_bytes"] == vis.nbytes
    finally:
        ops.release_buffers()


@pytest.mark.parametrize("chunk", [0, 5, L.CHUNKS_ADAPTIVE])
def test_imaging_cycles_equal_single_cycles(idg, chunk):
    """idg_imaging_cycles over three config-1 cycles with their own
    visibilities, the second on a plan that names only some rows (different
    plan and uvw buffers on the device): each cycle's grid and visibilities
    are those of the device-resident steps on its inputs, although each
    cycle's copies in ran during the cycle before it.  Then the bench's form:
    four cycles on one pair of host buffers."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config1()
    spec.aterm_sigma = 0.05
    obs = D.make_observation(spec)
    S, G, N = spec.subgrid_size, spec.grid_size, spec.n_subgrids
    gs = spec_for(G, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    keep = np.arange(N) % 3 != 1
    keep[0] = False
    plans = [obs.metadata, np.ascontiguousarray(obs.metadata[keep]), obs.metadata]
    vis = [_vis(spec, seed=s) for s in (51, 52, 53)]
    at = np.ascontiguousarray(obs.aterms)
    refs = []
    for md, v in zip(plans, vis):
        d = {k: dev(x) for k, x in dict(md=md, uvw=obs.uvw, k=obs.wavenumbers, vis=v, taper=obs.taper,
                                        at=obs.aterms).items()}
        sub = torch.empty((md.shape[0], 4, S, S), dtype=torch.complex64, device="cuda")
        g = torch.zeros((1, 4, G, G), dtype=torch.complex64, device="cuda")
        ops.grid_visibilities(gs, d["md"], d["uvw"], d["k"], d["vis"], d["taper"], d["at"], sub, g)
        vo = torch.zeros_like(d["vis"])
        ops.degrid_visibilities(gs, d["md"], d["uvw"], d["k"], vo, d["taper"], d["at"], sub, g)
        torch.cuda.synchronize()
        refs.append((g.cpu().numpy(), vo.cpu().numpy()))
    uvw = [obs.uvw.copy() for _ in plans]  # a buffer per cycle
    outs = [np.full(v.shape, np.nan + 1j * np.nan, np.complex64) for v in vis]
    grids = [np.zeros((1, 4, G, G), np.complex64) for _ in vis]
    try:
        ts = ops.imaging_cycles(gs, list(zip(plans, uvw, vis, outs, grids)), obs.wavenumbers, obs.taper, at,
                                chunk_subgrids=chunk)
        for i, ((g_ref, v_ref), md) in enumerate(zip(refs, plans)):
            named = np.zeros(vis[i].shape[0], bool)
            b0 = int(md["baseline_offset"][0])
            for m in md:
                r = int(m["baseline_offset"]) - b0 + int(m["time_offset"])
                named[r:r + int(m["nr_timesteps"])] = True
            check_rel(f"cycles[{i}] grid chunk={chunk}", grids[i], g_ref, TOL)
            check_rel(f"cycles[{i}] vis chunk={chunk}", outs[i][named], v_ref[named], TOL)
            assert np.all(outs[i][~named] == 0)
        assert all(t["total_ms"] > 0 and t["end_ms"] >= t["total_ms"] for t in ts)
        assert all(a["end_ms"] < b["end_ms"] for a, b in zip(ts, ts[1:]))
        assert ts[0]["h2d_bytes"] > ts[2]["h2d_bytes"]  # the constants travel with the first cycle only
        # four cycles on one pair of host buffers: each copies its inputs in
        # and its results out; the buffer ends with the last cycle's
        out = np.zeros_like(vis[0])
        ts = ops.imaging_cycles(gs, [(plans[0], uvw[0], vis[0], out)] * 4, obs.wavenumbers, obs.taper, at,
                                chunk_subgrids=chunk)
        check_rel(f"cycles x4 vis chunk={chunk}", out, refs[0][1], TOL)
        assert all(t["h2d_vis_bytes"] == vis[0].nbytes and t["d2h_vis_bytes"] == vis[0].nbytes for t in ts)
    finally:
        ops.release_buffers()


def test_degenerate_plan_entries_every_batched_shape(oracle_mod, idg):
    """Every batched launch shape on plan entries at the edges of what a plan may
    hold: zero and one timestep, empty and one-channel ranges, ranges starting
    at odd channels, subgrids at the grid's edges.  Gridder outputs equal the
    FP64 oracle (zeros where nothing is gridded); the degridder writes exactly
    the covered samples and leaves the others at zero."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops, tuning

    rng = np.random.default_rng(321)
    G, C, ns, S = 1024, 12, 4, 32
    image_size = 0.04
    spec = D.ObservationSpec(nstations=ns, disk_radius_m=2000.0, ntimesteps=64, timesteps_per_subgrid=64,
                             nchannels=C, f_start=140e6, f_end=170e6, subgrid_size=S, grid_size=G,
                             image_size=image_size, aterm_sigma=0.05, seed=11)
    obs = D.make_observation(spec)
    T = np.array([0, 1, 2, 3, 1, 5, 0, 7, 2, 1])
    lens = np.array([4, 0, 1, 12, 1, 3, 0, 2, 11, 1])
    c0 = np.array([0, 5, 11, 0, 7, 9, 3, 1, 1, 0])
    N = len(T)
    md = np.zeros(N, L.METADATA_DTYPE)
    md["time_offset"] = np.concatenate([[0], np.cumsum(T)[:-1]])
    md["nr_timesteps"] = T
    md["station1"] = rng.integers(0, ns - 1, N)
    md["station2"] = md["station1"] + 1
    md["x"] = np.array([0, G - S, 3, 17, G - S, 400, 0, 9, 511, G // 2 - S // 2])
    md["y"] = np.array([G - S, 0, 0, 500, G - S, 8, 0, 31, 2, G // 2 - S // 2])
    ext = np.zeros(N, L.SUBGRID_EXT_DTYPE)
    ext["channel_begin"] = c0
    ext["channel_end"] = c0 + lens
    rows = int(T.sum())
    uvw = np.ascontiguousarray(obs.uvw[:rows])
    vis = (rng.standard_normal((rows, C, 4)) + 1j * rng.standard_normal((rows, C, 4))).astype(np.complex64)
    sub_in = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    want_g, want_v = _oracle_with_ext(oracle_mod, G, S, ns, image_size, uvw, obs.wavenumbers, vis, obs.taper,
                                      obs.aterms, md, ext, sub_in)
    covered = np.zeros((rows, C), bool)
    for m, e in zip(md, ext):
        covered[m["time_offset"]:m["time_offset"] + m["nr_timesteps"], e["channel_begin"]:e["channel_end"]] = True
    empty = (T == 0) | (lens == 0)
    sp = spec_for(G, S, C, ns, obs.aterms.shape[0], image_size)
    ng, nd = tuning.num_shapes()
    saved = tuning.get_shapes(S)
    try:
        for sh in range(max(ng, nd)):
            g_sh, d_sh = min(sh, ng - 1), min(sh, nd - 1)
            tuning.set_shapes(S, g_sh, d_sh)
            got = grid_gpu(sp, md, uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, L.VARIANT_BATCHED, ext=ext)
            assert np.all(got[empty] == 0), g_sh
            check_rel(f"degenerate entries gridder shape {g_sh}", got[~empty], want_g[~empty], TOL)
            vg = degrid_gpu(sp, md, uvw, obs.wavenumbers, sub_in, obs.taper, obs.aterms, rows, L.VARIANT_BATCHED,
                            ext=ext)
            check_rel(f"degenerate entries degridder shape {d_sh}", vg[covered], want_v[covered], TOL)
            assert np.all(vg[~covered] == 0), d_sh
        assert ops.device_status(clear=True) == 0
    finally:
        tuning.set_shapes(S, *saved)
