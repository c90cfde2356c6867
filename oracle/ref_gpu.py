"""The reference's own GPU kernels, run as they are (TEST AND REFERENCE-ARM
INFRASTRUCTURE ONLY; never part of the product path).

``kernel_gridder_v7`` (gridding/src/gridding_benchmark.cu:231-246) and
``kernel_degridder_v6`` (gridding/src/degridding_benchmark.cu:106-203) are
compiled unmodified from the reference's sources into device-code cubins for
sm_103a (oracle/Makefile target ``ref``, or ``oracle.build()``), where those
sources are present.  This module loads the cubins with the CUDA driver API
(ctypes on libcuda) into the current context and launches them the way the
reference's GPU launchers do: one CTA of 128 threads per subgrid
(gridding_benchmark.cu:326-329, degridding_benchmark.cu:283).

The kernels check no bounds.  Before any launch the arguments are checked on
the host against the limits their index arithmetic implies (read from their
sources): S^2 a multiple of 512 for the gridder (4 pixels per thread, 128
threads, no pixel guard: gridding_benchmark.cu:77, :99-100), every subgrid's
timestep count a multiple of 128 for the degridder (its zeroing and sample
loops step by 128 without a guard: degridding_benchmark.cu:127-140, :165),
and every plan entry's rows, stations and A-term slot inside the arrays.
Calls outside those limits raise instead of launching.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GRIDDER_CUBIN = os.path.join(HERE, "_ref", "ref_gridder.cubin")
DEGRIDDER_CUBIN = os.path.join(HERE, "_ref", "ref_degridder.cubin")
THREADS = 128  # NUM_THREADS of both reference kernel files
# the kernels' symbols: namespace gridding_benchmark, (int, int, float, float,
# int, int, UVWCoordinate<float>*, float*, float2*, float*, float2*,
# Metadata*, float2*)
_SIG = "EiiffiiPNS_13UVWCoordinateIfEEPfP6float2S3_S5_PNS_8MetadataES5_"
GRIDDER_SYMBOL = "_ZN18gridding_benchmark17kernel_gridder_v7" + _SIG
DEGRIDDER_SYMBOL = "_ZN18gridding_benchmark19kernel_degridder_v6" + _SIG


def available() -> str | None:
    """None when both cubins are present, else why not."""
    missing = [p for p in (GRIDDER_CUBIN, DEGRIDDER_CUBIN) if not os.path.exists(p)]
    if missing:
        return "reference GPU kernels not built here (" + ", ".join(os.path.basename(m) for m in missing) + \
               " missing: the reference sources are not on this machine)"
    return None


class RefKernels:
    """The two reference kernels loaded into the calling thread's current
    CUDA context (create after the device is in use, e.g. by torch)."""

    def __init__(self):
        why = available()
        if why:
            raise RuntimeError(why)
        self._cu = ctypes.CDLL("libcuda.so.1")
        self._check(self._cu.cuInit(0), "cuInit")
        self._mods = []
        self.gridder_fn = self._load(GRIDDER_CUBIN, GRIDDER_SYMBOL)
        self.degridder_fn = self._load(DEGRIDDER_CUBIN, DEGRIDDER_SYMBOL)

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def _load(self, path: str, symbol: str) -> ctypes.c_void_p:
        mod = ctypes.c_void_p()
        self._check(self._cu.cuModuleLoad(ctypes.byref(mod), path.encode()), f"cuModuleLoad({os.path.basename(path)})")
        self._mods.append(mod)
        fn = ctypes.c_void_p()
        self._check(self._cu.cuModuleGetFunction(ctypes.byref(fn), mod, symbol.encode()), f"cuModuleGetFunction({symbol})")
        return fn

    def close(self):
        for m in self._mods:
            self._cu.cuModuleUnload(m)
        self._mods = []

    @staticmethod
    def check_plan(metadata: np.ndarray, nr_rows: int, nstations: int, nr_aterms: int, subgrid_size: int,
                   degridder: bool) -> None:
        """Raise ValueError unless every access of the kernels stays inside the arrays."""
        S = subgrid_size
        if (S * S) % (4 * THREADS):
            raise ValueError(f"kernel_gridder_v7 needs S^2 to be a multiple of 512 (S = {S})")
        md = metadata
        r0 = (md["baseline_offset"].astype(np.int64) - int(md["baseline_offset"][0])) + md["time_offset"]
        T = md["nr_timesteps"].astype(np.int64)
        if degridder and np.any(T % THREADS):
            raise ValueError("kernel_degridder_v6 needs every subgrid's timestep count to be a multiple of 128")
        if np.any(r0 < 0) or np.any(r0 + T > nr_rows) or np.any(T < 1):
            raise ValueError("a plan entry names rows outside the arrays")
        if np.any(md["station1"] >= nstations) or np.any(md["station2"] >= nstations):
            raise ValueError("a plan entry names a station outside the A-term table")
        if np.any(md["aterm_index"] < 0) or np.any(md["aterm_index"] >= nr_aterms):
            raise ValueError("a plan entry names an A-term slot outside the table")

    def _launch(self, fn, n_subgrids: int, grid_size: int, subgrid_size: int, image_size: float, w_step: float,
                nr_channels: int, nr_stations: int, uvw: int, wavenumbers: int, visibilities: int, spheroidal: int,
                aterms: int, metadata: int, subgrids: int, stream: int) -> None:
        vals = [ctypes.c_int(grid_size), ctypes.c_int(subgrid_size), ctypes.c_float(image_size),
                ctypes.c_float(w_step), ctypes.c_int(nr_channels), ctypes.c_int(nr_stations)]
        vals += [ctypes.c_void_p(p) for p in (uvw, wavenumbers, visibilities, spheroidal, aterms, metadata, subgrids)]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.addressof(v) for v in vals])
        self._check(self._cu.cuLaunchKernel(fn, ctypes.c_uint(n_subgrids), 1, 1, THREADS, 1, 1, 0,
                                            ctypes.c_void_p(stream), params, None), "cuLaunchKernel")

    def gridder(self, metadata: np.ndarray, nr_rows: int, nr_aterms: int, grid_size: int, subgrid_size: int,
                image_size: float, nr_channels: int, nr_stations: int, uvw: int, wavenumbers: int, visibilities: int,
                spheroidal: int, aterms: int, d_metadata: int, subgrids: int, stream: int = 0,
                w_step: float = 0.0, checked: bool = False) -> None:
        """subgrids <- kernel_gridder_v7; `metadata` is the host copy of the plan
        at `d_metadata` (checked once unless `checked`); pointers are device addresses."""
        if not checked:
            self.check_plan(metadata, nr_rows, nr_stations, nr_aterms, subgrid_size, degridder=False)
        self._launch(self.gridder_fn, metadata.shape[0], grid_size, subgrid_size, image_size, w_step, nr_channels,
                     nr_stations, uvw, wavenumbers, visibilities, spheroidal, aterms, d_metadata, subgrids, stream)

    def degridder(self, metadata: np.ndarray, nr_rows: int, nr_aterms: int, grid_size: int, subgrid_size: int,
                  image_size: float, nr_channels: int, nr_stations: int, uvw: int, wavenumbers: int, visibilities: int,
                  spheroidal: int, aterms: int, d_metadata: int, subgrids: int, stream: int = 0,
                  w_step: float = 0.0, checked: bool = False) -> None:
        """visibilities (the plan's rows) <- kernel_degridder_v6."""
        if not checked:
            self.check_plan(metadata, nr_rows, nr_stations, nr_aterms, subgrid_size, degridder=True)
        self._launch(self.degridder_fn, metadata.shape[0], grid_size, subgrid_size, image_size, w_step, nr_channels,
                     nr_stations, uvw, wavenumbers, visibilities, spheroidal, aterms, d_metadata, subgrids, stream)
