"""Serving: continuous batching of gridding and degridding jobs (idg_server_*).

``Server`` wraps the C ABI's scheduler: jobs are submitted from any thread
with host buffers, admitted as slots and HBM budget free up, run concurrently
on the GPU against device-resident uv-grids, and waited on with a bound.
``poisson_load`` drives a server with a Poisson stream of jobs of random
sizes and reports latency percentiles and throughput.
"""
from __future__ import annotations

import ctypes
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import IdgJob, IdgJobStats, IdgServerConfig, IdgServerSummary, ptr
from .ops import GridSpec


@dataclass
class JobData:
    """Host arrays of one job (keep them alive until the job is waited on):
    numpy arrays or CPU tensors; page-locked ones (pinned tensors) are copied
    without a staging pass."""

    spec: GridSpec
    metadata: np.ndarray
    uvw: object
    wavenumbers: object
    taper: object
    aterms: object
    vis: object              # gridding: input; degridding: output buffer (numpy or pinned tensor)
    ext: np.ndarray | None = None

    @property
    def nr_rows(self) -> int:
        return int(self.uvw.shape[0])

    @property
    def n_visibilities(self) -> int:
        T = self.metadata["nr_timesteps"].astype(np.int64)
        if self.ext is None:
            return int(T.sum() * self.spec.nr_channels)
        return int((T * (self.ext["channel_end"] - self.ext["channel_begin"])).sum())


class Server:
    def __init__(self, max_slots: int = 4, hbm_budget_bytes: int = 64 << 30, cta_share: bool = True):
        cfg = IdgServerConfig(max_slots, 1 if cta_share else 0, int(hbm_budget_bytes))
        h = ctypes.c_void_p()
        _lib.call("idg_server_create", ctypes.byref(cfg), ctypes.byref(h))
        self._h = h
        self._lock = threading.Lock()
        self._inflight: dict[int, tuple] = {}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().idg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid_create(self, grid_size: int, nr_w_planes: int = 1) -> int:
        g = ctypes.c_int64(0)
        _lib.call("idg_server_grid_create", self._h, int(grid_size), int(nr_w_planes), ctypes.byref(g))
        return int(g.value)

    def grid_read(self, grid_id: int, grid_size: int, nr_w_planes: int = 1) -> np.ndarray:
        out = np.empty((nr_w_planes, 4, grid_size, grid_size), np.complex64)
        _lib.call("idg_server_grid_read", self._h, int(grid_id), ptr(out))
        return out

    def grid_release(self, grid_id: int) -> None:
        _lib.call("idg_server_grid_release", self._h, int(grid_id))

    def submit(self, op: int, job: JobData, grid_id: int, variant: int = _lib.VARIANT_BATCHED) -> int:
        md = np.ascontiguousarray(job.metadata, dtype=_lib.METADATA_DTYPE)
        ext = None if job.ext is None else np.ascontiguousarray(job.ext, dtype=_lib.SUBGRID_EXT_DTYPE)
        j = IdgJob()
        j.op = op
        j.variant = variant
        j.params = job.spec.to_c()
        j.nr_subgrids = md.shape[0]
        j.metadata = ptr(md)
        j.ext = ptr(ext)
        j.nr_rows = job.nr_rows
        j.uvw = ptr(job.uvw)
        j.wavenumbers = ptr(job.wavenumbers)
        j.vis_in = ptr(job.vis) if op == _lib.IDG_JOB_GRID else None
        j.vis_out = ptr(job.vis) if op == _lib.IDG_JOB_DEGRID else None
        j.spheroidal = ptr(job.taper)
        j.aterms = ptr(job.aterms)
        j.grid_id = int(grid_id)
        jid = ctypes.c_int64(0)
        _lib.call("idg_server_submit", self._h, ctypes.byref(j), ctypes.byref(jid))
        with self._lock:
            self._inflight[int(jid.value)] = (job, md, ext)  # host buffers stay alive until waited on
        return int(jid.value)

    def wait(self, job_id: int, timeout_s: float = 600.0) -> dict:
        st = IdgJobStats()
        rc = _lib.load().idg_server_wait(self._h, int(job_id), int(timeout_s * 1000), ctypes.byref(st))
        if rc != _lib.IDG_ERR_TIMEOUT:
            with self._lock:
                self._inflight.pop(int(job_id), None)
        _lib.check(rc)
        return {"queue_ms": st.queue_ms, "run_ms": st.run_ms, "latency_ms": st.latency_ms,
                "visibilities": st.visibilities, "device_start_ms": st.device_start_ms,
                "device_end_ms": st.device_end_ms, "stream_start_ms": st.stream_start_ms,
                "stream_end_ms": st.stream_end_ms}

    def stats(self) -> dict:
        s = IdgServerSummary()
        _lib.call("idg_server_stats", self._h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in IdgServerSummary._fields_}


def poisson_load(server: Server, jobs: list[tuple[int, JobData, int]], rate_per_s: float, seed: int = 0,
                 timeout_s: float = 600.0) -> dict:
    """Submit `jobs` ((op, data, grid_id) in order) with exponential inter-arrival
    times of mean 1/rate, wait for all, and return the server statistics."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, len(jobs)) if rate_per_s > 0 else np.zeros(len(jobs))
    ids = []
    t0 = time.perf_counter()
    due = t0
    for (op, data, grid_id), gap in zip(jobs, gaps):
        due += gap
        delay = due - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        ids.append(server.submit(op, data, grid_id))
    per_job = [server.wait(i, timeout_s) for i in ids]
    wall = time.perf_counter() - t0
    s = server.stats()
    s["wall_s"] = wall
    s["jobs"] = per_job
    return s
