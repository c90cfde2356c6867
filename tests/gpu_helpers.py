"""Shared helpers for the GPU tests: upload host arrays, run the kernels
through the C ABI, bring results back."""
import numpy as np
import torch

import idg_gb300._lib as L
from idg_gb300 import ops


def dev(a, device="cuda"):
    if a.dtype == L.METADATA_DTYPE:
        return ops.metadata_tensor(a, device)
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def spec_for(G, S, C, ns, n_aterms, image_size, w_step=0.0, flags=0, W=1):
    return ops.GridSpec(grid_size=G, subgrid_size=S, nr_channels=C, nr_stations=ns, nr_aterms=n_aterms,
                        nr_w_planes=W, image_size=image_size, w_step=w_step, flags=flags)


def grid_gpu(spec, metadata, uvw, k, vis, taper, aterms, variant=L.VARIANT_PLAIN, ext=None):
    N = metadata.shape[0]
    S = spec.subgrid_size
    out = torch.empty((N, 4, S, S), dtype=torch.complex64, device="cuda")
    ops.gridder(spec, dev(metadata), dev(uvw), dev(k), dev(vis), dev(taper) if taper is not None else None,
                dev(aterms), out, variant=variant, ext=ops.ext_tensor(ext, "cuda") if ext is not None else None)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def degrid_gpu(spec, metadata, uvw, k, subgrids, taper, aterms, n_rows, variant=L.VARIANT_PLAIN, ext=None):
    vis = torch.zeros((n_rows, spec.nr_channels, 4), dtype=torch.complex64, device="cuda")
    ops.degridder(spec, dev(metadata), dev(uvw), dev(k), vis, dev(taper) if taper is not None else None,
                  dev(aterms), dev(np.ascontiguousarray(subgrids, np.complex64)), variant=variant,
                  ext=ops.ext_tensor(ext, "cuda") if ext is not None else None)
    torch.cuda.synchronize()
    return vis.cpu().numpy()
