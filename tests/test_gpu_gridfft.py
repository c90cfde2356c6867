"""The uv-grid FFT (idg_grid_fft), the imaging step after the adder.

* Against its definition evaluated in FP64 with numpy (both directions, with
  and without the separable grid correction), relative RMS <= 2e-6.
* Sizes 64 to 2048 cover every pass sequence of the radix-16 row transform
  (a last pass of radix 4, 8, none or 2).
* Round trip at 4096^2 and 8192^2: image -> uv after uv -> image gives G^2
  times the input (a size-independent property of the unnormalised pair).
"""
import numpy as np
import pytest
import torch

from conftest import check_rel
from gpu_helpers import spec_for

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _want(g, c, direction):
    G = g.shape[-1]
    x = np.arange(G) - G // 2
    E = np.exp(-2j * np.pi * np.outer(x, x) / G)  # E[u][x]
    cc = np.outer(c, c) if c is not None else 1.0
    if direction < 0:
        return cc * (E.T @ g @ E)
    return np.conj(E) @ (cc * g) @ np.conj(E).T


@pytest.mark.parametrize("G", [64, 128, 256, 512, 2048])
def test_grid_fft_matches_its_definition(idg, G):
    from idg_gb300 import ops

    rng = np.random.default_rng(G)
    grid = (rng.standard_normal((1, 4, G, G)) + 1j * rng.standard_normal((1, 4, G, G))).astype(np.complex64)
    corr = (1.0 + 0.2 * rng.standard_normal(G)).astype(np.float32)
    sp = spec_for(G, 32, 16, 4, 1, 0.05)
    for direction in (-1, 1):
        for c in (None, corr):
            d = torch.from_numpy(grid).cuda()
            ops.grid_fft(sp, d, direction, None if c is None else torch.from_numpy(c).cuda())
            torch.cuda.synchronize()
            got = d.cpu().numpy()
            want = np.stack([_want(grid[0, p].astype(np.complex128), None if c is None else c.astype(np.float64),
                                   direction) for p in range(4)])[None]
            check_rel(f"grid fft G={G} dir={direction} corr={c is not None}", got, want, TOL)


@pytest.mark.parametrize("G", [4096, 8192])
def test_grid_fft_round_trip(idg, G):
    from idg_gb300 import ops

    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    grid = torch.view_as_complex(torch.randn(4 * G * G * 2, generator=g, device="cuda").view(-1, 2)).view(1, 4, G, G)
    ref = grid.clone()
    sp = spec_for(G, 32, 16, 4, 1, 0.05)
    ops.grid_fft(sp, grid, -1)
    ops.grid_fft(sp, grid, +1)
    torch.cuda.synchronize()
    err = float(torch.linalg.vector_norm(grid / (G * G) - ref) / torch.linalg.vector_norm(ref))
    print(f"[parity] grid fft round trip G={G}: relative RMS {err:.3e} (tolerance {TOL})")
    assert err <= TOL
