"""Autotuner of the batched kernels' launch shapes, with an on-disk cache.

The batched gridder and degridder are compiled in several launch shapes
(threads per CTA, pixel pairs per thread, staging-tile size, CTAs per SM).
``autotune`` times every shape on a sample of the caller's plan and data
through ``idg_autotune`` (C ABI), which also selects the fastest for the
subgrid size on the current device; the choice is stored in a JSON cache
keyed by device name, subgrid size and channel count, and ``apply_cached``
re-selects it in a later process without timing again.
"""
from __future__ import annotations

import ctypes
import json
import os

import torch

from . import _lib
from ._lib import ptr
from .ops import GridSpec, _check_common, _req, _stream_handle


def cache_path() -> str:
    return os.environ.get("IDG_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "idg_gb300", "shapes.json"))


def _key(spec: GridSpec) -> str:
    return f"{torch.cuda.get_device_name()}|S={spec.subgrid_size}|C={spec.nr_channels}"


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only costs re-tuning next time


def num_shapes() -> tuple[int, int]:
    g, d = ctypes.c_int(0), ctypes.c_int(0)
    _lib.call("idg_batched_shapes", ctypes.byref(g), ctypes.byref(d))
    return g.value, d.value


def set_shapes(subgrid_size: int, gridder_shape: int, degridder_shape: int) -> None:
    _lib.call("idg_set_batched_shapes", subgrid_size, gridder_shape, degridder_shape)


def get_shapes(subgrid_size: int) -> tuple[int, int]:
    g, d = ctypes.c_int(0), ctypes.c_int(0)
    _lib.call("idg_get_batched_shapes", subgrid_size, ctypes.byref(g), ctypes.byref(d))
    return g.value, d.value


def apply_cached(spec: GridSpec) -> dict | None:
    """Select the cached shapes for this device / subgrid size / channel count, if any."""
    entry = _load().get(_key(spec))
    if entry:
        set_shapes(spec.subgrid_size, int(entry["gridder"]), int(entry["degridder"]))
    return entry


def autotune(spec: GridSpec, metadata, uvw, wavenumbers, vis, taper, aterms, subgrids, vis_out, ext=None,
             repeats: int = 2, stream=None, store: bool = True) -> dict:
    """Time every shape on this (device) sample and select the fastest; returns the timings."""
    _check_common(spec, metadata, uvw, wavenumbers, vis, taper, aterms)
    N, S = metadata.shape[0], spec.subgrid_size
    _req(subgrids, "subgrids", torch.complex64, (N, 4, S, S))
    _req(vis_out, "vis_out", torch.complex64, tuple(vis.shape))
    ng, nd = num_shapes()
    gms = (ctypes.c_double * ng)()
    dms = (ctypes.c_double * nd)()
    bg, bd = ctypes.c_int(0), ctypes.c_int(0)
    p = spec.to_c()
    _lib.call("idg_autotune", ctypes.byref(p), N, ptr(metadata), ptr(ext), uvw.shape[0], ptr(uvw), ptr(wavenumbers),
              ptr(vis), ptr(taper), ptr(aterms), ptr(subgrids), ptr(vis_out), _stream_handle(stream), int(repeats),
              gms, dms, ctypes.byref(bg), ctypes.byref(bd))
    result = {"gridder": bg.value, "degridder": bd.value, "gridder_ms": list(gms), "degridder_ms": list(dms),
              "sample_subgrids": N}
    if store:
        d = _load()
        d[_key(spec)] = result
        _store(d)
    return result
