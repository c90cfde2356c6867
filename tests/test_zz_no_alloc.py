"""idg_gridder_noalloc: the batched gridder for callers that may not allocate
device memory (for example an application whose own pool owns all of it, or a
processing loop that must not allocate once running).  Its scratch lives in a
static device array of the library, so the call allocates nothing.

Checked through the C ABI against idg_gridder(IDG_VARIANT_BATCHED) on the
same inputs, within the parity tolerance of the other tests, on two calls in a
row (the second call must start from a cleared work counter), with the
device's free memory unchanged across the second call.  A rejected plan entry
is reported by idg_noalloc_status().  This file is collected last so that a
failure here leaves every other test already run; it also passes when run
alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from idg_gb300 import ops

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _inputs():
    from idg_gb300 import datasets as D

    spec = D.config1()
    spec.aterm_sigma = 0.05
    obs = D.make_observation(spec)
    rng = np.random.default_rng(21)
    vis = (rng.standard_normal((spec.n_rows, spec.nchannels, 4)) +
           1j * rng.standard_normal((spec.n_rows, spec.nchannels, 4))).astype(np.complex64)
    dev = "cuda"
    t = dict(
        md=ops.metadata_tensor(obs.metadata, dev),
        uvw=torch.from_numpy(obs.uvw).to(dev),
        k=torch.from_numpy(obs.wavenumbers).to(dev),
        vis=torch.from_numpy(vis).to(dev),
        taper=torch.from_numpy(obs.taper).to(dev),
        at=torch.from_numpy(obs.aterms).to(dev),
    )
    gs = ops.GridSpec(spec.grid_size, spec.subgrid_size, spec.nchannels, spec.nstations, obs.aterms.shape[0], 1,
                      spec.image_size)
    return spec, gs, t


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_gridder_matches_batched_gridder():
    lib = L.load()
    spec, gs, t = _inputs()
    N, S = spec.n_subgrids, spec.subgrid_size
    ref = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    ops.gridder(gs, t["md"], t["uvw"], t["k"], t["vis"], t["taper"], t["at"], ref, variant=L.VARIANT_BATCHED)
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    p = gs.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    # the one-time set-up alone (an empty plan): address lookup, kernel loading
    rc = lib.idg_gridder_noalloc(ctypes.byref(p), 0, None, None, 0, None, None, None, None, None, None, stream)
    assert rc == L.IDG_OK, L.last_error()
    outs = [torch.full((N, 4, S, S), float("nan"), dtype=torch.complex64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    for call, out in enumerate(outs):
        free0 = torch.cuda.mem_get_info()[0]
        rc = lib.idg_gridder_noalloc(ctypes.byref(p), N, t["md"].data_ptr(), None, spec.n_rows, t["uvw"].data_ptr(),
                                     t["k"].data_ptr(), t["vis"].data_ptr(), t["taper"].data_ptr(),
                                     t["at"].data_ptr(), out.data_ptr(), stream)
        assert rc == L.IDG_OK, L.last_error()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        print(f"[noalloc] call {call}: device free memory {free0} -> {free1} bytes")
        if call == 1:
            # the first launch of a kernel may still reserve local memory for it;
            # a second call must take nothing
            assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
        st = ctypes.c_uint32(1 << 31)
        assert lib.idg_noalloc_status(stream, ctypes.byref(st)) == L.IDG_OK, L.last_error()
        assert st.value == 0
        got = out.cpu().numpy()
        assert np.isfinite(got.view(np.float32)).all(), f"call {call}: subgrids left unwritten"
        e = _rel(got, want)
        print(f"[parity] noalloc gridder call {call}: relative RMS {e:.3e} vs idg_gridder batched")
        assert e <= TOL


def test_noalloc_gridder_rejects_oversized_plan():
    lib = L.load()
    p = L.IdgParams(1024, 32, 16, 4, 1, 1, 0.05, 0.0, 0, 0)
    rc = lib.idg_gridder_noalloc(ctypes.byref(p), (1 << 30) + 1, None, None, 0, None, None, None, None, None, None,
                                 None)
    assert rc == L.IDG_ERR_UNSUPPORTED
    assert "2^30" in L.last_error() or "1073741824" in L.last_error()


def test_noalloc_status_reports_a_rejected_entry():
    """A plan entry naming a station outside the A-term table yields a zero
    subgrid and bit 0 of idg_noalloc_status(); the next good call clears it."""
    lib = L.load()
    spec, gs, t = _inputs()
    N, S = spec.n_subgrids, spec.subgrid_size
    md_np = t["md"].cpu().numpy().copy()
    bad = md_np.view(L.METADATA_DTYPE).reshape(-1)
    bad["station1"][1] = spec.nstations  # out of range
    md_bad = torch.from_numpy(md_np).cuda()
    p = gs.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    out = torch.full((N, 4, S, S), float("nan"), dtype=torch.complex64, device="cuda")
    for md, want in ((md_bad, 1), (t["md"], 0)):
        rc = lib.idg_gridder_noalloc(ctypes.byref(p), N, md.data_ptr(), None, spec.n_rows, t["uvw"].data_ptr(),
                                     t["k"].data_ptr(), t["vis"].data_ptr(), t["taper"].data_ptr(),
                                     t["at"].data_ptr(), out.data_ptr(), stream)
        assert rc == L.IDG_OK, L.last_error()
        st = ctypes.c_uint32(0)
        assert lib.idg_noalloc_status(stream, ctypes.byref(st)) == L.IDG_OK, L.last_error()
        assert st.value & 1 == want
        if want:
            assert np.abs(out[1].cpu().numpy()).max() == 0
