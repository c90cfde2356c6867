"""Failure detection on the GPU without faulting it.

The only device-side waits are the bounded mbarrier waits of the batched
gridders and of the grid FFT's row kernel on their bulk copies.  With
IDG_FLAG_TEST_LOST_COPY a kernel declares its first copy 16 bytes larger than
what it copies, so the wait runs out (after 2 s): the kernel sets bit 2 of the
device check word and stops, with no trap, bad address or endless loop.
These tests check that the host reads that status, and that the context stays
usable: the next call without the flag gives the right answer.
"""
import time

import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from conftest import check_rel
from gpu_helpers import dev, grid_gpu, spec_for
from test_gpu_gridfft import _want

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.mark.parametrize("shape", [13, 22])
def test_gridder_lost_copy_is_reported_and_the_context_recovers(oracle_mod, idg, shape):
    from idg_gb300 import datasets as D
    from idg_gb300 import ops, tuning

    spec = D.config1()
    obs = D.make_observation(spec)
    rng = np.random.default_rng(5)
    vis = (rng.standard_normal((spec.n_rows, spec.nchannels, 4)) +
           1j * rng.standard_normal((spec.n_rows, spec.nchannels, 4))).astype(np.complex64)
    S = spec.subgrid_size
    args = (spec.grid_size, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    saved = tuning.get_shapes(S)
    try:
        tuning.set_shapes(S, shape, saved[1])
        ops.device_status(clear=True)
        t0 = time.perf_counter()
        grid_gpu(spec_for(*args, flags=L.IDG_FLAG_TEST_LOST_COPY), obs.metadata, obs.uvw, obs.wavenumbers, vis,
                 obs.taper, obs.aterms, L.VARIANT_BATCHED)
        waited = time.perf_counter() - t0
        status = ops.device_status(clear=True)
        print(f"[failure] gridder shape {shape}: status {status:#x} after {waited:.1f} s")
        assert status & 4 and waited >= 1.5
        prm = oracle_mod.params(spec.grid_size, S, spec.nchannels, spec.nstations, spec.n_subgrids, spec.image_size)
        want = oracle_mod.gridder(prm, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms, obs.metadata)
        got = grid_gpu(spec_for(*args), obs.metadata, obs.uvw, obs.wavenumbers, vis, obs.taper, obs.aterms,
                       L.VARIANT_BATCHED)
        check_rel(f"gridder shape {shape} after a lost copy", got, want, TOL)
        assert ops.device_status(clear=True) == 0
    finally:
        tuning.set_shapes(S, *saved)


def test_grid_fft_lost_copy_is_reported_and_the_context_recovers(idg):
    from idg_gb300 import ops

    G = 64
    rng = np.random.default_rng(6)
    grid = (rng.standard_normal((1, 4, G, G)) + 1j * rng.standard_normal((1, 4, G, G))).astype(np.complex64)
    ops.device_status(clear=True)
    d = dev(grid)
    t0 = time.perf_counter()
    ops.grid_fft(spec_for(G, 32, 16, 4, 1, 0.05, flags=L.IDG_FLAG_TEST_LOST_COPY), d, -1)
    status = ops.device_status(clear=True)
    waited = time.perf_counter() - t0
    print(f"[failure] grid FFT: status {status:#x} after {waited:.1f} s")
    assert status & 4 and waited >= 1.5
    d = dev(grid)
    ops.grid_fft(spec_for(G, 32, 16, 4, 1, 0.05), d, -1)
    torch.cuda.synchronize()
    want = np.stack([_want(grid[0, p].astype(np.complex128), None, -1) for p in range(4)])[None]
    check_rel("grid fft after a lost copy", d.cpu().numpy(), want, 2e-6)
    assert ops.device_status(clear=True) == 0
