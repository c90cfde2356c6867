"""ctypes binding of ``libidg_gb300.so`` (declarations in include/idg_gb300.h).

The library is the only compute path: there is no Python or PyTorch
fallback.  If it is missing it is built in-tree on first use; if it cannot be
built or loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

IDG_OK = 0
IDG_ERR_INVALID_ARGUMENT = 1
IDG_ERR_CUDA = 2
IDG_ERR_OUT_OF_MEMORY = 3
IDG_ERR_UNSUPPORTED = 4
IDG_ERR_TIMEOUT = 5
IDG_ERR_DEVICE_CHECK = 6
IDG_ERR_NOT_FOUND = 7
IDG_ERR_REJECTED = 8

IDG_FLAG_DEGRID_ATERM_REFCPU = 0x1
IDG_FLAG_NO_TAPER = 0x2
IDG_FLAG_TEST_LOST_COPY = 0x100

VARIANT_PLAIN = 0
VARIANT_BATCHED = 1

# 36-byte plan entry (gridding/inc/types.hpp:17-25)
METADATA_DTYPE = np.dtype(
    [
        ("baseline_offset", "<i4"),
        ("time_offset", "<i4"),
        ("nr_timesteps", "<i4"),
        ("aterm_index", "<i4"),
        ("station1", "<u4"),
        ("station2", "<u4"),
        ("x", "<i4"),
        ("y", "<i4"),
        ("z", "<i4"),
    ]
)
SUBGRID_EXT_DTYPE = np.dtype([("channel_begin", "<i4"), ("channel_end", "<i4")])


class IdgParams(ctypes.Structure):
    _fields_ = [
        ("grid_size", ctypes.c_int32),
        ("subgrid_size", ctypes.c_int32),
        ("nr_channels", ctypes.c_int32),
        ("nr_stations", ctypes.c_int32),
        ("nr_aterms", ctypes.c_int32),
        ("nr_w_planes", ctypes.c_int32),
        ("image_size", ctypes.c_float),
        ("w_step", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("reserved", ctypes.c_int32),
    ]


class IdgPlannerParams(ctypes.Structure):
    _fields_ = [
        ("nr_baselines", ctypes.c_int64),
        ("nr_timesteps", ctypes.c_int32),
        ("nr_channels", ctypes.c_int32),
        ("subgrid_size", ctypes.c_int32),
        ("grid_size", ctypes.c_int32),
        ("max_timesteps", ctypes.c_int32),
        ("aterm_interval", ctypes.c_int32),
        ("margin", ctypes.c_int32),
        ("nr_w_planes", ctypes.c_int32),
        ("image_size", ctypes.c_double),
        ("w_step", ctypes.c_double),
    ]


class IdgBenchmarkResult(ctypes.Structure):
    _fields_ = [
        ("in_transfer_time", ctypes.c_double),
        ("out_transfer_time", ctypes.c_double),
        ("in_bandwidth", ctypes.c_double),
        ("out_bandwidth", ctypes.c_double),
        ("compute_time", ctypes.c_double),
    ]


class IdgCycleTiming(ctypes.Structure):
    _fields_ = [
        ("total_ms", ctypes.c_double),
        ("gridding_ms", ctypes.c_double),
        ("degridding_ms", ctypes.c_double),
        ("h2d_bytes", ctypes.c_int64),
        ("d2h_bytes", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("h2d_vis_ms", ctypes.c_double),
        ("d2h_vis_ms", ctypes.c_double),
        ("h2d_vis_bytes", ctypes.c_int64),
        ("d2h_vis_bytes", ctypes.c_int64),
        ("grid_chunks", ctypes.c_int64),
        ("degrid_chunks", ctypes.c_int64),
        ("gridding_wait_ms", ctypes.c_double),
        ("chunk_ratio", ctypes.c_double),
        ("end_ms", ctypes.c_double),
        ("h2d_span_ms", ctypes.c_double),
    ]


class IdgCycleIo(ctypes.Structure):
    _fields_ = [
        ("nr_subgrids", ctypes.c_int64),
        ("metadata", ctypes.c_void_p),
        ("nr_rows", ctypes.c_int64),
        ("uvw", ctypes.c_void_p),
        ("visibilities_in", ctypes.c_void_p),
        ("visibilities_out", ctypes.c_void_p),
        ("grid_out", ctypes.c_void_p),
        ("timing", ctypes.POINTER(IdgCycleTiming)),
    ]


CHUNKS_AUTO = -1  # IDG_CHUNKS_AUTO: idg_imaging_cycle sizes its chunks for the copy pipeline
CHUNKS_ADAPTIVE = -2  # IDG_CHUNKS_ADAPTIVE: ... with the growth ratio learned from the previous cycle


class IdgServerConfig(ctypes.Structure):
    _fields_ = [("max_slots", ctypes.c_int32), ("cta_share", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64)]


class IdgJob(ctypes.Structure):
    _fields_ = [
        ("op", ctypes.c_int32),
        ("variant", ctypes.c_int32),
        ("params", IdgParams),
        ("nr_subgrids", ctypes.c_int64),
        ("metadata", ctypes.c_void_p),
        ("ext", ctypes.c_void_p),
        ("nr_rows", ctypes.c_int64),
        ("uvw", ctypes.c_void_p),
        ("wavenumbers", ctypes.c_void_p),
        ("vis_in", ctypes.c_void_p),
        ("vis_out", ctypes.c_void_p),
        ("spheroidal", ctypes.c_void_p),
        ("aterms", ctypes.c_void_p),
        ("grid_id", ctypes.c_int64),
    ]


class IdgJobStats(ctypes.Structure):
    _fields_ = [
        ("queue_ms", ctypes.c_double),
        ("run_ms", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
        ("visibilities", ctypes.c_int64),
        ("status", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("device_start_ms", ctypes.c_double),
        ("device_end_ms", ctypes.c_double),
        ("stream_start_ms", ctypes.c_double),
        ("stream_end_ms", ctypes.c_double),
    ]


class IdgServerSummary(ctypes.Structure):
    _fields_ = [
        ("completed", ctypes.c_int64),
        ("rejected", ctypes.c_int64),
        ("failed", ctypes.c_int64),
        ("queued", ctypes.c_int64),
        ("running", ctypes.c_int64),
        ("hbm_in_use", ctypes.c_int64),
        ("hbm_peak", ctypes.c_int64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("mvis_per_s", ctypes.c_double),
    ]


IDG_JOB_GRID = 0
IDG_JOB_DEGRID = 1


class IdgLaunchConfig(ctypes.Structure):
    _fields_ = [
        ("niterations", ctypes.c_int64),
        ("grid_size", ctypes.c_int64),
        ("subgrid_size", ctypes.c_int64),
        ("nstations", ctypes.c_int64),
        ("nchannels", ctypes.c_int64),
        ("ntimeslots", ctypes.c_int64),
        ("ntimesteps_per_subgrid", ctypes.c_int64),
        ("image_size", ctypes.c_float),
        ("w_step", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("variant", ctypes.c_int32),
    ]


class IdgError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"idg error {code}: {message}")
        self.code = code


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int

# name -> argtypes (all entry points return int status unless listed in _RESTYPES)
_SIGNATURES = {
    "idg_abi_version": [],
    "idg_last_error": [],
    "idg_device_status": [_P, ctypes.POINTER(ctypes.c_uint32), _I32],
    "idg_gridder": [ctypes.POINTER(IdgParams), _I32, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P],
    "idg_gridder_noalloc": [ctypes.POINTER(IdgParams), _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P],
    "idg_noalloc_status": [_P, ctypes.POINTER(ctypes.c_uint32)],
    "idg_degridder": [ctypes.POINTER(IdgParams), _I32, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P],
    "idg_subgrid_fft": [ctypes.POINTER(IdgParams), _I64, _I32, _P, _P, _P],
    "idg_adder": [ctypes.POINTER(IdgParams), _I64, _P, _P, _P, _P],
    "idg_splitter": [ctypes.POINTER(IdgParams), _I64, _P, _P, _P, _P],
    "idg_split_subgrid_fft": [ctypes.POINTER(IdgParams), _I64, _P, _P, _P, _P, _P],
    "idg_tile_bins_create": [ctypes.POINTER(IdgParams), _I64, _P, ctypes.POINTER(ctypes.c_void_p)],
    "idg_tile_bins_destroy": [_P],
    "idg_tile_bins_info": [_P, ctypes.POINTER(ctypes.c_int64)],
    "idg_adder_binned": [_P, _P, _P, _P],
    "idg_grid_fft": [ctypes.POINTER(IdgParams), _P, _I32, _P, _P],
    "idg_grid_visibilities": [ctypes.POINTER(IdgParams), _I32, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P],
    "idg_degrid_visibilities": [ctypes.POINTER(IdgParams), _I32, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P],
    "idg_imaging_cycle": [ctypes.POINTER(IdgParams), _I32, _I64, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _I64,
                          ctypes.c_void_p],
    "idg_imaging_cycles": [ctypes.POINTER(IdgParams), _I32, _I64, ctypes.POINTER(IdgCycleIo), _P, _P, _P, _I64],
    "idg_release_buffers": [],
    "idg_plan_subgrids": [ctypes.POINTER(IdgPlannerParams), _P, _P, _P, _I64, _P, _P, ctypes.POINTER(ctypes.c_int64),
                          _P],
    "idg_plan_create": [ctypes.POINTER(IdgParams), _I32, _I64, _P, _P, _I64, ctypes.POINTER(ctypes.c_void_p)],
    "idg_plan_destroy": [_P],
    "idg_plan_set_cta_limit": [_P, _I32],
    "idg_plan_grid": [_P, _P, _P, _P, _P, _P, _P, _P],
    "idg_plan_degrid": [_P, _P, _P, _P, _P, _P, _P, _P],
    "idg_plan_capture_cycle": [_P, _P, _P, _P, _P, _P, _P, _P],
    "idg_plan_launch_cycle": [_P, _P],
    "idg_plan_status": [_P, _P, ctypes.POINTER(ctypes.c_uint32), _I32],
    "idg_cycle_capture": [_I32, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                          ctypes.POINTER(_P), ctypes.POINTER(_P), _P, ctypes.POINTER(_P), ctypes.POINTER(_P)],
    "idg_cycle_launch": [_P, _P],
    "idg_cycle_destroy": [_P],
    "idg_server_create": [ctypes.POINTER(IdgServerConfig), ctypes.POINTER(ctypes.c_void_p)],
    "idg_server_destroy": [_P],
    "idg_server_grid_create": [_P, _I32, _I32, ctypes.POINTER(ctypes.c_int64)],
    "idg_server_grid_read": [_P, _I64, _P],
    "idg_server_grid_release": [_P, _I64],
    "idg_server_submit": [_P, ctypes.POINTER(IdgJob), ctypes.POINTER(ctypes.c_int64)],
    "idg_server_wait": [_P, _I64, _I64, ctypes.POINTER(IdgJobStats)],
    "idg_server_stats": [_P, ctypes.POINTER(IdgServerSummary)],
    "idg_gridding_launch": [ctypes.POINTER(IdgLaunchConfig), _P, _P, _P, _P, _P, _P, _P, _P, _P,
                            ctypes.POINTER(IdgBenchmarkResult)],
    "idg_degridding_launch": [ctypes.POINTER(IdgLaunchConfig), _P, _P, _P, _P, _P, _P, _P, _P, _P,
                              ctypes.POINTER(IdgBenchmarkResult)],
    "idg_reference_dataset": [_I64, _I64, _I64, _I64, _I64, _I64, ctypes.c_float, _P, _P, _P, _P, _P, _P, _P, _P],
    "idg_measure_fp32_peak": [ctypes.POINTER(ctypes.c_double)],
    "idg_batched_shapes": [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "idg_set_batched_shapes": [_I32, _I32, _I32],
    "idg_get_batched_shapes": [_I32, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "idg_autotune": [ctypes.POINTER(IdgParams), _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32,
                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                     ctypes.POINTER(ctypes.c_int)],
}
_RESTYPES = {"idg_last_error": ctypes.c_char_p, "idg_abi_version": ctypes.c_int}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the native library; raises if impossible."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if not os.path.exists(path):
            if not build_if_missing:
                raise IdgError(IDG_ERR_UNSUPPORTED, f"{path} is missing and building was not requested")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, argtypes in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def last_error() -> str:
    msg = load().idg_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    if rc != IDG_OK:
        raise IdgError(rc, last_error())


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def ptr(x) -> int | None:
    """Raw address of a torch tensor (device or host) or numpy array; None for None."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr()
    if isinstance(x, int):
        return x
    raise TypeError(f"cannot take the address of {type(x)}")
