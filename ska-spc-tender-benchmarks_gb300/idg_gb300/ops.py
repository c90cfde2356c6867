"""Device-level IDG operations on CUDA tensors, through the C ABI.

Each function validates shapes and dtypes on the host and calls the matching
``idg_*`` entry point on the tensor's device and the current (or given)
stream.  Layouts are those of include/idg_gb300.h.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import IdgParams, ptr

VARIANT_PLAIN = _lib.VARIANT_PLAIN
VARIANT_BATCHED = _lib.VARIANT_BATCHED


@dataclass
class GridSpec:
    """Geometry and physics of one gridding problem (idg_params)."""

    grid_size: int
    subgrid_size: int
    nr_channels: int
    nr_stations: int
    nr_aterms: int = 1
    nr_w_planes: int = 1
    image_size: float = 0.1
    w_step: float = 0.0
    flags: int = 0

    def to_c(self) -> IdgParams:
        return IdgParams(self.grid_size, self.subgrid_size, self.nr_channels, self.nr_stations, self.nr_aterms,
                         self.nr_w_planes, self.image_size, self.w_step, self.flags, 0)


def _stream_handle(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _req(t: torch.Tensor, name: str, dtype, shape=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")


def metadata_tensor(md: np.ndarray, device) -> torch.Tensor:
    """Plan entries (METADATA_DTYPE) as an int32 [N, 9] device tensor."""
    md = np.ascontiguousarray(md, dtype=_lib.METADATA_DTYPE)
    return torch.from_numpy(md.view(np.int32).reshape(-1, 9).copy()).to(device)


def ext_tensor(ext: np.ndarray | None, device) -> torch.Tensor | None:
    if ext is None:
        return None
    ext = np.ascontiguousarray(ext, dtype=_lib.SUBGRID_EXT_DTYPE)
    return torch.from_numpy(ext.view(np.int32).reshape(-1, 2).copy()).to(device)


def _check_common(spec: GridSpec, metadata, uvw, wavenumbers, vis, taper, aterms):
    _req(metadata, "metadata", torch.int32)
    if metadata.dim() != 2 or metadata.shape[1] != 9:
        raise ValueError("metadata must be [N, 9] int32 (36-byte entries)")
    _check_data(spec, uvw, wavenumbers, vis, taper, aterms)


def _check_data(spec: GridSpec, uvw, wavenumbers, vis, taper, aterms):
    _req(uvw, "uvw", torch.float32)
    if uvw.dim() != 2 or uvw.shape[1] != 3:
        raise ValueError("uvw must be [rows, 3] float32")
    _req(wavenumbers, "wavenumbers", torch.float32, (spec.nr_channels,))
    _req(vis, "visibilities", torch.complex64, (uvw.shape[0], spec.nr_channels, 4))
    S = spec.subgrid_size
    if taper is not None:
        _req(taper, "spheroidal", torch.float32, (S, S))
    _req(aterms, "aterms", torch.complex64, (spec.nr_aterms, spec.nr_stations, S, S, 4))


def gridder(spec: GridSpec, metadata, uvw, wavenumbers, vis, taper, aterms, subgrids, variant=VARIANT_PLAIN,
            ext=None, stream=None):
    """subgrids[N,4,S,S] complex64 <- gridder(vis)."""
    _check_common(spec, metadata, uvw, wavenumbers, vis, taper, aterms)
    N, S = metadata.shape[0], spec.subgrid_size
    _req(subgrids, "subgrids", torch.complex64, (N, 4, S, S))
    if ext is not None:
        _req(ext, "ext", torch.int32, (N, 2))
    p = spec.to_c()
    _lib.call("idg_gridder", ctypes.byref(p), variant, N, ptr(metadata), ptr(ext), uvw.shape[0], ptr(uvw),
              ptr(wavenumbers), ptr(vis), ptr(taper), ptr(aterms), ptr(subgrids), _stream_handle(stream))
    return subgrids


def degridder(spec: GridSpec, metadata, uvw, wavenumbers, vis, taper, aterms, subgrids, variant=VARIANT_PLAIN,
              ext=None, stream=None):
    """vis[rows named by the plan] <- degridder(subgrids)."""
    _check_common(spec, metadata, uvw, wavenumbers, vis, taper, aterms)
    N, S = metadata.shape[0], spec.subgrid_size
    _req(subgrids, "subgrids", torch.complex64, (N, 4, S, S))
    if ext is not None:
        _req(ext, "ext", torch.int32, (N, 2))
    p = spec.to_c()
    _lib.call("idg_degridder", ctypes.byref(p), variant, N, ptr(metadata), ptr(ext), uvw.shape[0], ptr(uvw),
              ptr(wavenumbers), ptr(vis), ptr(taper), ptr(aterms), ptr(subgrids), _stream_handle(stream))
    return vis


def subgrid_fft(spec: GridSpec, subgrids, direction: int, taper=None, stream=None):
    """In-place FFT of subgrids[N,4,S,S]; direction +1 image->uv, -1 uv->image."""
    S = spec.subgrid_size
    _req(subgrids, "subgrids", torch.complex64)
    if subgrids.dim() != 4 or subgrids.shape[1:] != (4, S, S):
        raise ValueError("subgrids must be [N, 4, S, S]")
    if taper is not None:
        _req(taper, "taper", torch.float32, (S, S))
    p = spec.to_c()
    _lib.call("idg_subgrid_fft", ctypes.byref(p), subgrids.shape[0], int(direction), ptr(taper), ptr(subgrids),
              _stream_handle(stream))
    return subgrids


def adder(spec: GridSpec, metadata, subgrids, grid, stream=None):
    S, G, W = spec.subgrid_size, spec.grid_size, spec.nr_w_planes
    _req(metadata, "metadata", torch.int32)
    _req(subgrids, "subgrids", torch.complex64, (metadata.shape[0], 4, S, S))
    _req(grid, "grid", torch.complex64, (W, 4, G, G))
    p = spec.to_c()
    _lib.call("idg_adder", ctypes.byref(p), metadata.shape[0], ptr(metadata), ptr(subgrids), ptr(grid),
              _stream_handle(stream))
    return grid


class TileBins:
    """The adder with a fixed summation order (idg_tile_bins_* / idg_adder_binned):
    bins made once from a plan's host metadata; ``add`` sums the plan's
    subgrids into a grid in the same order on every call, so the grid is
    reproducible bit for bit."""

    def __init__(self, spec: GridSpec, metadata: np.ndarray):
        md = np.ascontiguousarray(metadata, dtype=_lib.METADATA_DTYPE)
        self.spec = spec
        self.nr_subgrids = md.shape[0]
        p = spec.to_c()
        h = ctypes.c_void_p()
        _lib.call("idg_tile_bins_create", ctypes.byref(p), md.shape[0], ptr(md), ctypes.byref(h))
        self._h = h

    def info(self) -> dict:
        v = (ctypes.c_int64 * 4)()
        _lib.call("idg_tile_bins_info", self._h, v)
        return {"work_items": v[0], "multi_chunk_tiles": v[1], "partial_tiles": v[2], "partial_bytes": v[3]}

    def add(self, subgrids, grid, stream=None):
        S, G, W = self.spec.subgrid_size, self.spec.grid_size, self.spec.nr_w_planes
        _req(subgrids, "subgrids", torch.complex64, (self.nr_subgrids, 4, S, S))
        _req(grid, "grid", torch.complex64, (W, 4, G, G))
        _lib.call("idg_adder_binned", self._h, ptr(subgrids), ptr(grid), _stream_handle(stream))
        return grid

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().idg_tile_bins_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def splitter(spec: GridSpec, metadata, grid, subgrids, stream=None):
    S, G, W = spec.subgrid_size, spec.grid_size, spec.nr_w_planes
    _req(metadata, "metadata", torch.int32)
    _req(subgrids, "subgrids", torch.complex64, (metadata.shape[0], 4, S, S))
    _req(grid, "grid", torch.complex64, (W, 4, G, G))
    p = spec.to_c()
    _lib.call("idg_splitter", ctypes.byref(p), metadata.shape[0], ptr(metadata), ptr(grid), ptr(subgrids),
              _stream_handle(stream))
    return subgrids


def split_subgrid_fft(spec: GridSpec, metadata, grid, subgrids, taper=None, stream=None):
    """splitter followed by subgrid_fft(-1, taper), in one pass over the data."""
    S, G, W = spec.subgrid_size, spec.grid_size, spec.nr_w_planes
    _req(metadata, "metadata", torch.int32)
    _req(subgrids, "subgrids", torch.complex64, (metadata.shape[0], 4, S, S))
    _req(grid, "grid", torch.complex64, (W, 4, G, G))
    if taper is not None:
        _req(taper, "taper", torch.float32, (S, S))
    p = spec.to_c()
    _lib.call("idg_split_subgrid_fft", ctypes.byref(p), metadata.shape[0], ptr(metadata), ptr(grid), ptr(taper),
              ptr(subgrids), _stream_handle(stream))
    return subgrids


def grid_fft(spec: GridSpec, grid, direction: int, correction=None, stream=None):
    """In-place 2-D FFT of every plane of grid[W,4,G,G] (idg_grid_fft): direction -1
    uv -> image with the grid correction applied after, +1 image -> uv with it before."""
    G, W = spec.grid_size, spec.nr_w_planes
    _req(grid, "grid", torch.complex64, (W, 4, G, G))
    if correction is not None:
        _req(correction, "correction", torch.float32, (G,))
    p = spec.to_c()
    _lib.call("idg_grid_fft", ctypes.byref(p), ptr(grid), int(direction), ptr(correction), _stream_handle(stream))
    return grid


def grid_visibilities(spec: GridSpec, metadata, uvw, wavenumbers, vis, taper, aterms, subgrids, grid,
                      variant=VARIANT_BATCHED, ext=None, stream=None):
    """Gridding step: gridder -> subgrid FFT (+1, taper) -> adder; accumulates into grid[W,4,G,G]."""
    _check_common(spec, metadata, uvw, wavenumbers, vis, taper, aterms)
    N, S, G, W = metadata.shape[0], spec.subgrid_size, spec.grid_size, spec.nr_w_planes
    _req(subgrids, "subgrids", torch.complex64, (N, 4, S, S))
    _req(grid, "grid", torch.complex64, (W, 4, G, G))
    p = spec.to_c()
    _lib.call("idg_grid_visibilities", ctypes.byref(p), variant, N, ptr(metadata), ptr(ext), uvw.shape[0], ptr(uvw),
              ptr(wavenumbers), ptr(vis), ptr(taper), ptr(aterms), ptr(subgrids), ptr(grid), _stream_handle(stream))
    return grid


def degrid_visibilities(spec: GridSpec, metadata, uvw, wavenumbers, vis, taper, aterms, subgrids, grid,
                        variant=VARIANT_BATCHED, ext=None, stream=None):
    """Degridding step: splitter -> subgrid FFT (-1, taper) -> degridder into vis."""
    _check_common(spec, metadata, uvw, wavenumbers, vis, taper, aterms)
    N, S, G, W = metadata.shape[0], spec.subgrid_size, spec.grid_size, spec.nr_w_planes
    _req(subgrids, "subgrids", torch.complex64, (N, 4, S, S))
    _req(grid, "grid", torch.complex64, (W, 4, G, G))
    p = spec.to_c()
    _lib.call("idg_degrid_visibilities", ctypes.byref(p), variant, N, ptr(metadata), ptr(ext), uvw.shape[0],
              ptr(uvw), ptr(wavenumbers), ptr(vis), ptr(taper), ptr(aterms), ptr(subgrids), ptr(grid),
              _stream_handle(stream))
    return vis


def imaging_cycle(spec: GridSpec, metadata: np.ndarray, uvw: np.ndarray, wavenumbers: np.ndarray, vis_in, taper,
                  aterms, vis_out, grid_out=None, variant=VARIANT_BATCHED, chunk_subgrids=0) -> dict:
    """One grid + degrid cycle on HOST buffers (numpy arrays or pinned CPU tensors) through idg_imaging_cycle."""
    md = np.ascontiguousarray(metadata, dtype=_lib.METADATA_DTYPE)
    for name, a in (("uvw", uvw), ("wavenumbers", wavenumbers), ("taper", taper)):
        if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]):
            raise TypeError(f"{name} must be a C-contiguous float32 numpy array")
    t = _lib.IdgCycleTiming()
    p = spec.to_c()
    _lib.call("idg_imaging_cycle", ctypes.byref(p), variant, md.shape[0], ptr(md), uvw.shape[0], ptr(uvw),
              ptr(wavenumbers), ptr(vis_in), ptr(taper), ptr(aterms), ptr(vis_out), ptr(grid_out),
              int(chunk_subgrids), ctypes.byref(t))
    return {f: getattr(t, f) for f, _ in _lib.IdgCycleTiming._fields_}


def imaging_cycles(spec: GridSpec, cycles, wavenumbers: np.ndarray, taper, aterms, variant=VARIANT_BATCHED,
                   chunk_subgrids=0) -> list[dict]:
    """Several grid + degrid cycles on HOST buffers through idg_imaging_cycles,
    each cycle's copies in running while the cycle before it degrids.
    `cycles`: a sequence of (metadata, uvw, vis_in, vis_out) or (metadata,
    uvw, vis_in, vis_out, grid_out) tuples.  Returns one timing dict per cycle."""
    for name, a in (("wavenumbers", wavenumbers), ("taper", taper)):
        if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]):
            raise TypeError(f"{name} must be a C-contiguous float32 numpy array")
    keep, ios, timings = [], (_lib.IdgCycleIo * max(1, len(cycles)))(), []
    for i, c in enumerate(cycles):
        metadata, uvw, vis_in, vis_out = c[:4]
        grid_out = c[4] if len(c) > 4 else None
        md = np.ascontiguousarray(metadata, dtype=_lib.METADATA_DTYPE)
        if not (isinstance(uvw, np.ndarray) and uvw.dtype == np.float32 and uvw.flags["C_CONTIGUOUS"]):
            raise TypeError(f"cycle {i}: uvw must be a C-contiguous float32 numpy array")
        t = _lib.IdgCycleTiming()
        keep.append(md)
        timings.append(t)
        ios[i] = _lib.IdgCycleIo(md.shape[0], ptr(md), uvw.shape[0], ptr(uvw), ptr(vis_in), ptr(vis_out),
                                 ptr(grid_out), ctypes.pointer(t))
    p = spec.to_c()
    _lib.call("idg_imaging_cycles", ctypes.byref(p), variant, len(cycles), ios, ptr(wavenumbers), ptr(taper),
              ptr(aterms), int(chunk_subgrids))
    return [{f: getattr(t, f) for f, _ in _lib.IdgCycleTiming._fields_} for t in timings]


def plan_subgrids(uvw, frequencies, baselines, nr_timesteps: int, subgrid_size: int, grid_size: int,
                  image_size: float, max_timesteps: int, aterm_interval: int = 0, margin: int | None = None,
                  capacity: int | None = None, w_step: float = 0.0, nr_w_planes: int = 1, stream=None):
    """The uvw-driven plan with channel and time splitting, computed on the GPU
    (idg_plan_subgrids): uvw [rows, 3] float32, frequencies [C] float64 and
    baselines [nb, 2] int32/uint32 on the device.  Returns (metadata, ext) as
    numpy arrays, identical to datasets.plan_subgrids_split on the same inputs."""
    nb = baselines.shape[0]
    if uvw.shape != (nb * nr_timesteps, 3) or uvw.dtype != torch.float32 or not uvw.is_cuda:
        raise ValueError("uvw must be a float32 CUDA tensor [nr_baselines * nr_timesteps, 3]")
    if frequencies.dtype != torch.float64 or not frequencies.is_cuda:
        raise ValueError("frequencies must be a float64 CUDA tensor")
    if baselines.dtype not in (torch.int32,) or not baselines.is_cuda or baselines.shape[1] != 2:
        raise ValueError("baselines must be an int32 CUDA tensor [nr_baselines, 2]")
    prm = _lib.IdgPlannerParams(nb, nr_timesteps, frequencies.shape[0], subgrid_size, grid_size, max_timesteps,
                                aterm_interval, subgrid_size // 4 if margin is None else margin, nr_w_planes,
                                image_size, float(np.float32(w_step)))
    n = ctypes.c_int64(0)
    cap = capacity if capacity is not None else 0
    if cap == 0:  # counting call: learn the size, then plan into exactly that much
        rc = _lib.load().idg_plan_subgrids(ctypes.byref(prm), ptr(uvw), ptr(frequencies), ptr(baselines), 0, None,
                                            None, ctypes.byref(n), _stream_handle(stream))
        if rc not in (_lib.IDG_OK, _lib.IDG_ERR_INVALID_ARGUMENT) or n.value <= 0:
            _lib.check(rc)
        cap = int(n.value)
    md = torch.empty((cap, 9), dtype=torch.int32, device=uvw.device)
    ext = torch.empty((cap, 2), dtype=torch.int32, device=uvw.device)
    _lib.call("idg_plan_subgrids", ctypes.byref(prm), ptr(uvw), ptr(frequencies), ptr(baselines), cap, ptr(md),
              ptr(ext), ctypes.byref(n), _stream_handle(stream))
    k = int(n.value)
    md_np = md[:k].cpu().numpy().copy().view(_lib.METADATA_DTYPE).reshape(-1)
    ext_np = ext[:k].cpu().numpy().copy().view(_lib.SUBGRID_EXT_DTYPE).reshape(-1)
    return md_np, ext_np


class Plan:
    """A device-resident execution plan (idg_plan_*): metadata, longest-first work
    list and subgrid work space on the device; optional CUDA graph of one cycle."""

    def __init__(self, spec: GridSpec, metadata: np.ndarray, nr_rows: int, ext: np.ndarray | None = None,
                 variant: int = VARIANT_BATCHED):
        self.spec = spec
        self._md = np.ascontiguousarray(metadata, dtype=_lib.METADATA_DTYPE)
        self._ext = None if ext is None else np.ascontiguousarray(ext, dtype=_lib.SUBGRID_EXT_DTYPE)
        self.nr_subgrids = int(self._md.shape[0])
        self.nr_rows = int(nr_rows)
        self._p = spec.to_c()
        h = ctypes.c_void_p()
        _lib.call("idg_plan_create", ctypes.byref(self._p), variant, self.nr_subgrids, ptr(self._md), ptr(self._ext),
                  self.nr_rows, ctypes.byref(h))
        self._h = h
        self._keep = None

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().idg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cta_limit(self, max_ctas: int) -> None:
        _lib.call("idg_plan_set_cta_limit", self._h, int(max_ctas))

    def _check(self, uvw, wavenumbers, vis, taper, aterms, grid):
        _check_data(self.spec, uvw, wavenumbers, vis, taper, aterms)
        S, G, W = self.spec.subgrid_size, self.spec.grid_size, self.spec.nr_w_planes
        _req(grid, "grid", torch.complex64, (W, 4, G, G))
        if uvw.shape[0] != self.nr_rows:
            raise ValueError(f"uvw has {uvw.shape[0]} rows, the plan was built for {self.nr_rows}")

    def grid(self, uvw, wavenumbers, vis, taper, aterms, grid, stream=None):
        self._check(uvw, wavenumbers, vis, taper, aterms, grid)
        _lib.call("idg_plan_grid", self._h, ptr(uvw), ptr(wavenumbers), ptr(vis), ptr(taper), ptr(aterms), ptr(grid),
                  _stream_handle(stream))
        return grid

    def degrid(self, uvw, wavenumbers, vis_out, taper, aterms, grid, stream=None):
        self._check(uvw, wavenumbers, vis_out, taper, aterms, grid)
        _lib.call("idg_plan_degrid", self._h, ptr(uvw), ptr(wavenumbers), ptr(vis_out), ptr(taper), ptr(aterms),
                  ptr(grid), _stream_handle(stream))
        return vis_out

    def capture_cycle(self, uvw, wavenumbers, vis_in, taper, aterms, grid, vis_out):
        """Capture zero-grid + grid + degrid on these buffers as a CUDA graph."""
        self._check(uvw, wavenumbers, vis_in, taper, aterms, grid)
        _req(vis_out, "vis_out", torch.complex64, tuple(vis_in.shape))
        _lib.call("idg_plan_capture_cycle", self._h, ptr(uvw), ptr(wavenumbers), ptr(vis_in), ptr(taper), ptr(aterms),
                  ptr(grid), ptr(vis_out))
        self._keep = (uvw, wavenumbers, vis_in, taper, aterms, grid, vis_out)  # the graph holds raw addresses

    def launch_cycle(self, stream=None):
        _lib.call("idg_plan_launch_cycle", self._h, _stream_handle(stream))

    def status(self, clear: bool = True, stream=None) -> int:
        v = ctypes.c_uint32(0)
        _lib.call("idg_plan_status", self._h, _stream_handle(stream), ctypes.byref(v), 1 if clear else 0)
        return int(v.value)


class Cycle:
    """One imaging cycle over several plans sharing one uv-grid (idg_cycle_*),
    captured as a single CUDA graph: zero the grid, grid with every plan, then
    degrid with every plan.  `parts` holds, per plan, the device tensors
    (uvw, wavenumbers, vis_in, taper, aterms, vis_out)."""

    def __init__(self, plans: list, parts: list, grid):
        if len(plans) != len(parts) or not plans:
            raise ValueError("one (uvw, wavenumbers, vis_in, taper, aterms, vis_out) tuple per plan")
        for p, (uvw, k, vin, taper, at, vout) in zip(plans, parts):
            p._check(uvw, k, vin, taper, at, grid)
            _req(vout, "vis_out", torch.complex64, tuple(vin.shape))
        n = len(plans)
        arr = lambda xs: (ctypes.c_void_p * n)(*[ptr(x) for x in xs])
        h = ctypes.c_void_p()
        _lib.call("idg_cycle_capture", n, (ctypes.c_void_p * n)(*[p._h.value for p in plans]),
                  arr([q[0] for q in parts]), arr([q[1] for q in parts]), arr([q[2] for q in parts]),
                  arr([q[3] for q in parts]), arr([q[4] for q in parts]), ptr(grid), arr([q[5] for q in parts]),
                  ctypes.byref(h))
        self._h = h
        self._keep = (plans, parts, grid)  # the graph holds raw addresses

    def launch(self, stream=None) -> None:
        _lib.call("idg_cycle_launch", self._h, _stream_handle(stream))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().idg_cycle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def release_buffers() -> None:
    _lib.call("idg_release_buffers")


def device_status(clear: bool = True, stream=None) -> int:
    v = ctypes.c_uint32(0)
    _lib.call("idg_device_status", _stream_handle(stream), ctypes.byref(v), 1 if clear else 0)
    return int(v.value)


def measure_fp32_peak() -> float:
    f = ctypes.c_double(0)
    _lib.call("idg_measure_fp32_peak", ctypes.byref(f))
    return float(f.value)
