"""Properties of the CUDA gridder and degridder that need no oracle run, so
they hold at the full config-2 size (316,800 subgrids, 6.49e8 visibilities,
6.64e11 pixel-visibilities) where the FP64 oracle would take hours:

* a point source on a pixel centre grids to its known answer, T C
  exp(i phase_offset), at that pixel of every subgrid (both forms);
* the batched and plain forms agree at full size (relative RMS <= 1e-5 for
  the subgrids and the predicted visibilities);
* gridder and degridder are adjoint at full size: <G v, P> = <v, D P>
  (relative difference <= 1e-5), with the degridder's adjoint A-term
  convention and the taper on both sides.
"""
import numpy as np
import pytest
import torch

import idg_gb300._lib as L
from gpu_helpers import grid_gpu, spec_for
from test_oracle import _point_source

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.mark.parametrize("variant", [L.VARIANT_PLAIN, L.VARIANT_BATCHED])
def test_point_source_known_answer_gpu(idg, variant):
    from idg_gb300 import datasets as D

    spec = D.config1()
    obs = D.make_observation(spec)
    S = spec.subgrid_size
    px, py = S // 2 + 5, S // 2 - 7
    vis, want = _point_source(spec, obs, px, py)
    sp = spec_for(spec.grid_size, S, spec.nchannels, spec.nstations, obs.aterms.shape[0], spec.image_size)
    got = grid_gpu(sp, obs.metadata, obs.uvw, obs.wavenumbers, vis, np.ones((S, S), np.float32), obs.aterms, variant)
    for pol in range(4):
        err = np.max(np.abs(got[:, pol, py, px] - want) / np.abs(want))
        print(f"[known answer] variant {variant} pol {pol}: max relative error {err:.2e}")
        assert err <= TOL
    mag = np.abs(got[:, 0]).reshape(spec.n_subgrids, -1)
    assert np.all(mag.argmax(axis=1) == py * S + px)


def _vdot64(a: torch.Tensor, b: torch.Tensor, chunk: int = 1 << 26) -> complex:
    """sum(conj(a) * b) accumulated in complex128, in chunks of the flattened arrays."""
    a, b = a.reshape(-1), b.reshape(-1)
    tot = torch.zeros((), dtype=torch.complex128, device=a.device)
    for i in range(0, a.numel(), chunk):
        tot += torch.sum(a[i:i + chunk].to(torch.complex128).conj() * b[i:i + chunk].to(torch.complex128))
    return complex(tot.item())


def _rel_rms(x: torch.Tensor, ref: torch.Tensor, chunk: int = 1 << 26) -> float:
    x, ref = x.reshape(-1), ref.reshape(-1)
    num = den = 0.0
    for i in range(0, x.numel(), chunk):
        d = (x[i:i + chunk] - ref[i:i + chunk]).to(torch.complex128)
        num += float(torch.sum(d.real ** 2 + d.imag ** 2))
        r = ref[i:i + chunk].to(torch.complex128)
        den += float(torch.sum(r.real ** 2 + r.imag ** 2))
    return (num / den) ** 0.5


def test_config2_full_size_forms_agree_and_are_adjoint(idg):
    from idg_gb300 import datasets as D
    from idg_gb300 import ops

    spec = D.config2()
    obs = D.make_observation(spec)
    S, C, N = spec.subgrid_size, spec.nchannels, spec.n_subgrids
    dev = torch.device("cuda")
    md = ops.metadata_tensor(obs.metadata, dev)
    uvw = torch.from_numpy(obs.uvw).to(dev)
    k = torch.from_numpy(obs.wavenumbers).to(dev)
    taper = torch.from_numpy(obs.taper).to(dev)
    at = torch.from_numpy(obs.aterms).to(dev)
    vis = D.visibilities(spec, device=dev, seed=77)
    g = torch.Generator(device=dev)
    g.manual_seed(78)
    P = torch.complex(torch.randn((N, 4, S, S), generator=g, device=dev),
                      torch.randn((N, 4, S, S), generator=g, device=dev))
    sp = ops.GridSpec(spec.grid_size, S, C, spec.nstations, obs.aterms.shape[0], 1, spec.image_size, spec.w_step)
    out = {}
    for variant in (L.VARIANT_PLAIN, L.VARIANT_BATCHED):
        Gv = torch.empty((N, 4, S, S), dtype=torch.complex64, device=dev)
        ops.gridder(sp, md, uvw, k, vis, taper, at, Gv, variant=variant)
        DP = torch.zeros_like(vis)
        ops.degridder(sp, md, uvw, k, DP, taper, at, P, variant=variant)
        torch.cuda.synchronize()
        assert ops.device_status(clear=True) == 0
        lhs, rhs = _vdot64(Gv, P), _vdot64(vis, DP)
        rel = abs(lhs - rhs) / abs(lhs)
        print(f"[full size] variant {variant}: <Gv,P> = {lhs:.6e}, <v,DP> = {rhs:.6e}, relative difference {rel:.2e}")
        assert rel <= TOL
        out[variant] = (Gv, DP)
    eg = _rel_rms(out[L.VARIANT_BATCHED][0], out[L.VARIANT_PLAIN][0])
    ev = _rel_rms(out[L.VARIANT_BATCHED][1], out[L.VARIANT_PLAIN][1])
    print(f"[full size] batched vs plain: subgrids {eg:.2e}, visibilities {ev:.2e} relative RMS")
    assert eg <= TOL and ev <= TOL
