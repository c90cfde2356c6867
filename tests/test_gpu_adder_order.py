"""The adder with a fixed summation order (idg_tile_bins_* / idg_adder_binned)
and the paths that use it.

- Same definition as the FP64 oracle's adder (within 2e-6, the FFT/adder
  tolerance), w-planes with mirrored entries, entries outside the planes and
  footprints partly outside the grid included, added onto a grid that is not
  zero.
- Tiles with more than one chunk of subgrids (crowded footprints, as near the
  centre of a real uv-grid) go through the partial-tile pass.
- Two calls give the same grid bit for bit, and so do two runs of a plan's
  gridding step; the atomic idg_adder agrees within 1e-6.
"""
import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from conftest import check_rel
from gpu_helpers import dev, spec_for

pytestmark = pytest.mark.gpu


def _crowded(S, G, W, N, rng, spread):
    """N entries crowded into a few tiles round the grid centre, plus entries on
    the grid's edges, mirrored (negative z) and outside the w-planes."""
    md = np.zeros(N, L.METADATA_DTYPE)
    md["x"] = G // 2 - S // 2 + rng.integers(-spread, spread + 1, N)
    md["y"] = G // 2 - S // 2 + rng.integers(-spread, spread + 1, N)
    md["z"] = rng.integers(-W, W, N)
    md["x"][:6] = [-S + 3, G - 3, 0, G - S, -S, G]  # partly / wholly outside the grid
    md["y"][:6] = [5, 7, -S + 1, G - 2, 9, 11]
    md["z"][6] = W       # outside the planes: skipped
    md["z"][7] = -W - 1
    return md


@pytest.mark.parametrize("S,G,W,N,spread", [(16, 96, 2, 40, 30), (32, 256, 2, 900, 6), (24, 200, 1, 500, 40)])
def test_binned_adder_vs_oracle_and_repeatable(oracle_mod, idg, S, G, W, N, spread):
    from idg_gb300 import ops

    rng = np.random.default_rng(S * 1000 + N)
    md = _crowded(S, G, W, N, rng, spread)
    sub = (rng.standard_normal((N, 4, S, S)) + 1j * rng.standard_normal((N, 4, S, S))).astype(np.complex64)
    g0 = (rng.standard_normal((W, 4, G, G)) + 1j * rng.standard_normal((W, 4, G, G))).astype(np.complex64)
    sp = spec_for(G, S, 1, 2, 1, 0.05, W=W)
    bins = ops.TileBins(sp, md)
    info = bins.info()
    print(f"[adder] S={S} G={G} W={W} N={N}: {info}")
    if N >= 500:
        assert info["multi_chunk_tiles"] > 0 and info["partial_tiles"] > 0
    d_sub = dev(sub)
    grids = []
    for _ in range(2):
        grid = dev(g0)
        bins.add(d_sub, grid)
        torch.cuda.synchronize()
        grids.append(grid.cpu().numpy())
    assert np.array_equal(grids[0], grids[1]), "two calls gave different grids"
    want = oracle_mod.adder(sub, md, G, W, grid=g0)
    check_rel(f"binned adder S={S} N={N}", grids[0], want, 2e-6)
    atomic = dev(g0)
    ops.adder(sp, dev(md), d_sub, atomic)
    torch.cuda.synchronize()
    check_rel(f"binned vs atomic adder S={S} N={N}", grids[0], atomic.cpu().numpy(), 1e-6)
    bins.close()


def test_plan_gridding_step_is_repeatable(idg):
    """A plan's gridding step (gridder -> FFT -> binned adder) twice on the same
    data: the same grid bit for bit."""
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config2()
    obs = D.truncate_observation(D.make_observation(spec), 4096)
    spec = obs.spec
    gs = ops.GridSpec(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, obs.aterms.shape[0], 1,
                      spec.image_size)
    vis = D.visibilities(spec, device="cuda", seed=9)
    d = dict(uvw=torch.from_numpy(obs.uvw).cuda(), k=torch.from_numpy(obs.wavenumbers).cuda(),
             taper=torch.from_numpy(obs.taper).cuda(), at=torch.from_numpy(obs.aterms).cuda())
    plan = ops.Plan(gs, obs.metadata, spec.n_rows)
    out = []
    for _ in range(2):
        grid = torch.zeros((1, 4, spec.grid_size, spec.grid_size), dtype=torch.complex64, device="cuda")
        plan.grid(d["uvw"], d["k"], vis, d["taper"], d["at"], grid)
        torch.cuda.synchronize()
        out.append(grid.cpu().numpy())
    plan.close()
    assert np.abs(out[0]).max() > 0
    assert np.array_equal(out[0], out[1])
