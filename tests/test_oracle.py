"""The oracle against the reference's own outputs (golden fixtures) and against
independent definitions.  CPU only."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_rms

CASES = golden_cases()


def _params(O, d, image_size=0.1):
    G, S, ns, C, nts, T = d["cfg"]
    return O.params(G, S, C, ns, d["metadata"].shape[0], image_size, 0.0)


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.rsplit("/", 1)[-1])
def test_float_gridder_matches_reference_bit_for_bit(oracle_mod, path):
    O, d = oracle_mod, load_golden(path)
    prm = _params(O, d)
    out = O.gridder(prm, d["uvw"], d["wavenumbers"], d["vis"], d["spheroidal"], d["aterms"], d["metadata"], fp64=False)
    assert np.array_equal(out.view(np.uint32), d["gridder_out"].view(np.uint32))


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.rsplit("/", 1)[-1])
def test_float_degridder_matches_reference_bit_for_bit(oracle_mod, path):
    O, d = oracle_mod, load_golden(path)
    prm = _params(O, d)
    out = O.degridder(prm, d["uvw"], d["wavenumbers"], d["degridder_in"], d["spheroidal"], d["aterms"],
                      d["metadata"], d["vis"].shape[0], aterm_mode=O.ATERM_REFCPU, fp64=False)
    assert np.array_equal(out.view(np.uint32), d["degridder_out"].view(np.uint32))


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.rsplit("/", 1)[-1])
def test_fp64_oracle_close_to_reference(oracle_mod, path):
    # The reference computes in FP32 with phases of 1e3 rad that cancel: it sits
    # ~1e-4 (relative RMS) from the same sums in FP64.  The FP64 oracle must agree
    # with it to that level and no better is expected.
    O, d = oracle_mod, load_golden(path)
    prm = _params(O, d)
    g64 = O.gridder(prm, d["uvw"], d["wavenumbers"], d["vis"], d["spheroidal"], d["aterms"], d["metadata"])
    assert rel_rms(d["gridder_out"], g64) < 5e-4
    v64 = O.degridder(prm, d["uvw"], d["wavenumbers"], d["degridder_in"], d["spheroidal"], d["aterms"],
                      d["metadata"], d["vis"].shape[0], aterm_mode=O.ATERM_REFCPU)
    assert rel_rms(d["degridder_out"], v64) < 5e-4


def _naive_dft(P, direction, taper=None):
    S = P.shape[-1]
    k = np.arange(S) - S / 2
    xs = np.arange(S) - S / 2 + 0.5
    E = np.exp(direction * 2j * np.pi * np.outer(k, xs) / S)  # [k][x]
    if direction > 0:
        Pt = P * (taper if taper is not None else 1.0)
        return np.einsum("jy,ix,...yx->...ji", E, E, Pt)
    out = np.einsum("jy,ix,...ji->...yx", E, E, P)
    return out * (taper if taper is not None else 1.0)


@pytest.mark.parametrize("S", [8, 16, 24, 32])
def test_dft_oracle_matches_definition(oracle_mod, S):
    rng = np.random.default_rng(S)
    P = rng.standard_normal((2, 4, S, S)) + 1j * rng.standard_normal((2, 4, S, S))
    taper = rng.random((S, S)).astype(np.float32)
    for direction in (1, -1):
        got = oracle_mod.subgrid_dft(P, direction, taper)
        want = _naive_dft(P, direction, taper.astype(np.float64))
        assert np.allclose(got, want, rtol=1e-12, atol=1e-9)
    # round trip: backward(forward(P)) = S^2 P without taper
    rt = oracle_mod.subgrid_dft(oracle_mod.subgrid_dft(P, 1), -1)
    assert np.allclose(rt, S * S * P, rtol=1e-12, atol=1e-9)


def test_dft_adjoint(oracle_mod):
    S = 16
    rng = np.random.default_rng(0)
    a = rng.standard_normal((1, 4, S, S)) + 1j * rng.standard_normal((1, 4, S, S))
    b = rng.standard_normal((1, 4, S, S)) + 1j * rng.standard_normal((1, 4, S, S))
    lhs = np.vdot(oracle_mod.subgrid_dft(a, 1), b)
    rhs = np.vdot(a, oracle_mod.subgrid_dft(b, -1))
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)


def test_adder_splitter(oracle_mod):
    import idg_gb300._lib as L

    S, G = 8, 40
    md = np.zeros(4, L.METADATA_DTYPE)
    md["x"] = [0, 30, -3, 10]
    md["y"] = [0, 35, 5, 10]
    rng = np.random.default_rng(1)
    sub = rng.standard_normal((4, 4, S, S)) + 1j * rng.standard_normal((4, 4, S, S))
    grid = oracle_mod.adder(sub, md, G)
    want = np.zeros((1, 4, G, G), complex)
    for s in range(4):
        for j in range(S):
            for i in range(S):
                gy, gx = md["y"][s] + j, md["x"][s] + i
                if 0 <= gy < G and 0 <= gx < G:
                    want[0, :, gy, gx] += sub[s, :, j, i]
    assert np.allclose(grid, want)
    back = oracle_mod.splitter(grid, md[:1], S)
    assert np.allclose(back[0], grid[0, :, 0:S, 0:S])
    # adjointness: <adder(s), g> == <s, splitter(g)>
    g = rng.standard_normal((1, 4, G, G)) + 1j * rng.standard_normal((1, 4, G, G))
    assert abs(np.vdot(grid, g) - np.vdot(sub, oracle_mod.splitter(g, md, S))) < 1e-9 * abs(np.vdot(grid, g))


def test_gridder_degridder_adjoint_fp64(oracle_mod):
    """<G v, P> == <v, D P> with the adjoint A-term convention (FP64 oracle)."""
    import idg_gb300.datasets as D

    spec = D.config1()
    spec.nstations = 4
    spec.ntimesteps = spec.timesteps_per_subgrid = 16
    spec.nchannels = 4
    spec.aterm_sigma = 0.1
    obs = D.make_observation(spec)
    rng = np.random.default_rng(3)
    v = (rng.standard_normal((spec.n_rows, 4, 4)) + 1j * rng.standard_normal((spec.n_rows, 4, 4))).astype(np.complex64)
    S = spec.subgrid_size
    P = (rng.standard_normal((spec.n_subgrids, 4, S, S)) + 1j * rng.standard_normal((spec.n_subgrids, 4, S, S))).astype(np.complex64)
    prm = oracle_mod.params(spec.grid_size, S, spec.nchannels, spec.nstations, spec.n_subgrids, spec.image_size)
    Gv = oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, v, obs.taper, obs.aterms, obs.metadata)
    DP = oracle_mod.degridder(prm, obs.uvw, obs.wavenumbers, P, obs.taper, obs.aterms, obs.metadata, spec.n_rows,
                              aterm_mode=oracle_mod.ATERM_ADJOINT)
    lhs = np.vdot(Gv, P.astype(np.complex128))
    rhs = np.vdot(v.astype(np.complex128), DP)
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)


def _point_source(spec, obs, px, py):
    """Visibilities of a unit point source at the centre of subgrid pixel
    (px, py): V[t][c][pol] = exp(+i k_c (u l0 + v m0 + w n0)), the same in all
    four correlations, and the known answer at that pixel of every subgrid:
    T C exp(i phase_offset(l0, m0)) (identity A-terms, unit taper).  The image
    size is taken at float32 precision, as the gridders receive it."""
    S, G, img = spec.subgrid_size, spec.grid_size, float(np.float32(spec.image_size))
    l0 = (px + 0.5 - S / 2) * img / S
    m0 = (py + 0.5 - S / 2) * img / S
    n0 = (l0 * l0 + m0 * m0) / (1.0 + np.sqrt(1.0 - l0 * l0 - m0 * m0))
    uvw = obs.uvw.astype(np.float64)
    k = obs.wavenumbers.astype(np.float64)
    arg = (uvw[:, 0] * l0 + uvw[:, 1] * m0 + uvw[:, 2] * n0)[:, None] * k[None, :]
    vis = np.repeat(np.exp(1j * arg)[:, :, None], 4, axis=2).astype(np.complex64)
    md = obs.metadata
    u_off = (md["x"].astype(np.float64) + S / 2 - G / 2) * 2 * np.pi / img
    v_off = (md["y"].astype(np.float64) + S / 2 - G / 2) * 2 * np.pi / img
    want = md["nr_timesteps"] * spec.nchannels * np.exp(1j * (u_off * l0 + v_off * m0))
    return vis, want


def test_point_source_known_answer(oracle_mod):
    """A point source on a pixel centre grids to T C exp(i phase_offset) at that
    pixel in every subgrid and correlation, and every other pixel is smaller
    (FP64 oracle, config-1 geometry, identity A-terms, unit taper)."""
    import idg_gb300.datasets as D

    spec = D.config1()
    obs = D.make_observation(spec)
    S = spec.subgrid_size
    px, py = S // 2 + 5, S // 2 - 7
    vis, want = _point_source(spec, obs, px, py)
    prm = oracle_mod.params(spec.grid_size, S, spec.nchannels, spec.nstations, spec.n_subgrids, spec.image_size)
    ones = np.ones((S, S), np.float32)
    got = oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, vis, ones, obs.aterms, obs.metadata)
    for pol in range(4):
        assert np.max(np.abs(got[:, pol, py, px] - want) / np.abs(want)) < 1e-7
    mag = np.abs(got[:, 0]).reshape(spec.n_subgrids, -1)
    assert np.all(mag.argmax(axis=1) == py * S + px)
