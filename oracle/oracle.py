"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline /
reference arm import this module.  It loads

* ``oracle/_build/libidg_oracle.so`` -- the C restatement of the reference's
  CPU gridder/degridder (float, operation for operation) and its FP64 twin,
  plus FP64 DFT/adder/splitter definitions (``oracle/idg_oracle.c``);
* ``oracle/_ref/libidgref.so`` when present -- the reference's own CPU
  launchers and synthetic-input generators compiled from its sources
  (``oracle/Makefile`` target ``ref``; only buildable where the reference
  sources are present).
"""
from __future__ import annotations

import ctypes
import os
import re
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libidg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libidgref.so")
REF_GRIDDER_CUBIN = os.path.join(HERE, "_ref", "ref_gridder.cubin")
REF_DEGRIDDER_CUBIN = os.path.join(HERE, "_ref", "ref_degridder.cubin")


def _reference_dir() -> str:
    """Where the reference sources are: $IDG_REFERENCE_DIR when set, else the
    default that oracle/Makefile (the recipe that compiles them) gives
    IDG_REFERENCE_DIR; empty when neither names one."""
    env = os.environ.get("IDG_REFERENCE_DIR", "")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                m = re.match(r"\s*IDG_REFERENCE_DIR\s*\?=\s*(\S+)", line)
                if m:
                    return m.group(1)
    except OSError:
        pass
    return ""


REFERENCE_DIR = _reference_dir()

# 36-byte plan entry, gridding/inc/types.hpp:7-25
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
assert METADATA_DTYPE.itemsize == 36

ATERM_REFCPU = 0
ATERM_ADJOINT = 1


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("grid_size", ctypes.c_int),
        ("subgrid_size", ctypes.c_int),
        ("nr_channels", ctypes.c_int),
        ("nr_stations", ctypes.c_int),
        ("nr_subgrids", ctypes.c_int),
        ("image_size", ctypes.c_float),
        ("w_step", ctypes.c_float),
    ]


_FLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared"]


def _stale(target: str, deps: list[str]) -> bool:
    return not os.path.exists(target) or os.path.getmtime(target) < max(os.path.getmtime(d) for d in deps)


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and, where the reference sources exist, the reference bridge).

    Same commands as oracle/Makefile, run directly so that no make is needed."""
    src = [os.path.join(HERE, "idg_oracle.c"), os.path.join(HERE, "idg_oracle.h")]
    if _stale(ORACLE_SO, src):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.run(["gcc", "-std=gnu11", *_FLAGS, "-o", ORACLE_SO, src[0], "-lm"], check=True)
    for build_type in BUILD_FLAGS:  # the CPU baseline's other builds, compiled ahead of any timing
        if build_type != "-O2":
            _compile_variant(build_type)
    if with_ref is None:
        with_ref = bool(REFERENCE_DIR) and os.path.isdir(REFERENCE_DIR)
    if with_ref:
        g = os.path.join(REFERENCE_DIR, "gridding")
        ref_src = [os.path.join(g, "src", f) for f in ("gridding_benchmark.cpp", "degridding_benchmark.cpp",
                                                        "gridding_initialization.cpp")]
        bridge = os.path.join(HERE, "ref_bridge.cpp")
        inc = ["-I" + os.path.join(g, "inc"), "-I" + os.path.join(REFERENCE_DIR, "benchmarks-common", "inc")]
        if _stale(REF_SO, [bridge, *ref_src]):
            os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
            subprocess.run(["g++", "-std=c++17", *_FLAGS, "-DENABLE_OMP", "-DENABLE_CPU=1", "-w", *inc,
                            "-o", REF_SO, bridge, *ref_src, "-lm"], check=True)
        # the reference's GPU kernels, device code only (same command as the Makefile's)
        for cubin, src in ((REF_GRIDDER_CUBIN, "gridding_benchmark.cu"), (REF_DEGRIDDER_CUBIN, "degridding_benchmark.cu")):
            cu = os.path.join(g, "src", src)
            nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
            if os.path.exists(cu) and os.path.exists(nvcc) and _stale(cubin, [cu]):
                subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-cubin",
                                "-w", "-DENABLE_GPU=1", *inc, "-o", cubin, cu], check=True)


_lib = None
_ref = None
_variants: dict = {}

# Builds of the float restatement for the CPU baseline: the oracle's own -O2,
# -O3, and -O0 -g, the reference CMake's build type (gridding/CMakeLists.txt:37
# sets -g and no optimisation level).  -march/-mcpu=native is not used: the
# same flags must build on x86-64 and aarch64 hosts.
BUILD_FLAGS = {"-O2": ["-O2"], "-O3": ["-O3"], "-O0 -g": ["-O0", "-g"]}


def variant_lib(build: str = "-O2") -> ctypes.CDLL:
    """The oracle library compiled with one of BUILD_FLAGS (built on first use)."""
    if build == "-O2":
        return lib()
    if build not in _variants:
        _variants[build] = ctypes.CDLL(_compile_variant(build))
    return _variants[build]


def _compile_variant(build: str) -> str:
    tag = build.replace(" ", "").replace("-", "")
    path = os.path.join(HERE, "_build", f"libidg_oracle_{tag}.so")
    src = os.path.join(HERE, "idg_oracle.c")
    if _stale(path, [src, os.path.join(HERE, "idg_oracle.h")]):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        flags = [f for f in _FLAGS if f != "-O2"] + BUILD_FLAGS[build]
        subprocess.run(["gcc", "-std=gnu11", *flags, "-o", path, src, "-lm"], check=True)
    return path


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        _lib = ctypes.CDLL(ORACLE_SO)
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_SO)
        _ref.ref_cpu_gridding.restype = ctypes.c_double
        _ref.ref_cpu_degridding.restype = ctypes.c_double
    return _ref


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def params(grid_size, subgrid_size, nr_channels, nr_stations, nr_subgrids, image_size, w_step=0.0):
    return OracleParams(grid_size, subgrid_size, nr_channels, nr_stations, nr_subgrids, image_size, w_step)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def gridder(prm: OracleParams, uvw, wavenumbers, vis, spheroidal, aterms, metadata, fp64=True):
    """Returns subgrids [N][4][S][S] complex128 (fp64) or complex64 (float restatement)."""
    N, S = prm.nr_subgrids, prm.subgrid_size
    # converted arrays stay referenced by these locals for the whole call
    uvw_c = _f32(uvw)
    k_c = _f32(wavenumbers)
    vis_c = np.ascontiguousarray(vis, dtype=np.complex64)
    sph_c = _f32(spheroidal)
    at_c = np.ascontiguousarray(aterms, dtype=np.complex64)
    md_c = np.ascontiguousarray(metadata, dtype=METADATA_DTYPE)
    args = [ctypes.byref(prm), _p(uvw_c), _p(k_c), _p(vis_c), _p(sph_c), _p(at_c), _p(md_c)]
    if fp64:
        out = np.zeros((N, 4, S, S), dtype=np.complex128)
        lib().oracle_gridder_f64(*args, _p(out))
    else:
        out = np.zeros((N, 4, S, S), dtype=np.complex64)
        lib().oracle_gridder_f32(*args, _p(out))
    return out


def degridder(prm: OracleParams, uvw, wavenumbers, subgrids, spheroidal, aterms, metadata, nr_rows,
              aterm_mode=ATERM_ADJOINT, fp64=True):
    """Returns vis [nr_rows][C][4] (complex128 or complex64); rows not covered stay 0."""
    C = prm.nr_channels
    uvw_c = _f32(uvw)
    k_c = _f32(wavenumbers)
    sub_c = np.ascontiguousarray(subgrids, dtype=np.complex64)
    sph_c = _f32(spheroidal)
    at_c = np.ascontiguousarray(aterms, dtype=np.complex64)
    md_c = np.ascontiguousarray(metadata, dtype=METADATA_DTYPE)
    if fp64:
        out = np.zeros((nr_rows, C, 4), dtype=np.complex128)
        fn = lib().oracle_degridder_f64
    else:
        out = np.zeros((nr_rows, C, 4), dtype=np.complex64)
        fn = lib().oracle_degridder_f32
    fn(ctypes.byref(prm), ctypes.c_int(aterm_mode), _p(uvw_c), _p(k_c), _p(sub_c), _p(sph_c), _p(at_c), _p(md_c), _p(out))
    return out


def subgrid_dft(subgrids, direction, taper=None):
    """FP64 DFT of complex subgrids [N][4][S][S] (see idg_oracle.h for the definition)."""
    a = np.ascontiguousarray(subgrids, dtype=np.complex128)
    N, _, S, _ = a.shape
    out = np.zeros_like(a)
    t = _f32(taper) if taper is not None else None
    lib().oracle_subgrid_dft_f64(ctypes.c_int(N), ctypes.c_int(S), ctypes.c_int(direction),
                                 _p(t) if t is not None else None, _p(a), _p(out))
    return out


def adder(subgrids, metadata, grid_size, nr_w_planes=1, grid=None):
    a = np.ascontiguousarray(subgrids, dtype=np.complex128)
    N, _, S, _ = a.shape
    g = np.zeros((nr_w_planes, 4, grid_size, grid_size), np.complex128) if grid is None else np.ascontiguousarray(grid, np.complex128).copy()
    md = np.ascontiguousarray(metadata, dtype=METADATA_DTYPE)
    lib().oracle_adder_f64(ctypes.c_int(N), ctypes.c_int(S), ctypes.c_int(grid_size), ctypes.c_int(nr_w_planes), _p(md), _p(a), _p(g))
    return g


def splitter(grid, metadata, subgrid_size):
    g = np.ascontiguousarray(grid, dtype=np.complex128)
    W, _, G, _ = g.shape
    md = np.ascontiguousarray(metadata, dtype=METADATA_DTYPE)
    N = md.shape[0]
    out = np.zeros((N, 4, subgrid_size, subgrid_size), np.complex128)
    lib().oracle_splitter_f64(ctypes.c_int(N), ctypes.c_int(subgrid_size), ctypes.c_int(G), ctypes.c_int(W), _p(md), _p(g), _p(out))
    return out


def omp_threads() -> int:
    return int(lib().oracle_omp_max_threads())


def cpu_gridding_omp(prm, uvw, wavenumbers, vis, spheroidal, aterms, metadata, out, build: str = "-O2"):
    """Timed CPU baseline (float restatement of the reference's OMP launcher). Writes into `out`."""
    return variant_lib(build).oracle_cpu_gridding_omp(ctypes.byref(prm), _p(uvw), _p(wavenumbers), _p(vis),
                                                      _p(spheroidal), _p(aterms), _p(metadata), _p(out))


def cpu_degridding_omp(prm, uvw, wavenumbers, subgrids, spheroidal, aterms, metadata, out, build: str = "-O2"):
    return variant_lib(build).oracle_cpu_degridding_omp(ctypes.byref(prm), _p(uvw), _p(wavenumbers), _p(subgrids),
                                                        _p(spheroidal), _p(aterms), _p(metadata), _p(out))


# ---------------------------------------------------------------------------
# reference bridge (only where oracle/_ref was built)
# ---------------------------------------------------------------------------
def ref_dataset(grid_size, subgrid_size, nstations, nchannels, ntimeslots, ntimesteps):
    """The reference's own synthetic inputs (srand(0) sequence of gridding_benchmark.cpp:203-213)."""
    nb = nstations * (nstations - 1) // 2
    nsg = nb * ntimeslots
    T, C, S = ntimesteps, nchannels, subgrid_size
    d = dict(
        uvw=np.zeros((nsg * T, 3), np.float32),
        frequencies=np.zeros(C, np.float32),
        wavenumbers=np.zeros(C, np.float32),
        vis=np.zeros((nsg * T, C, 4), np.complex64),
        baselines=np.zeros((nb, 2), np.uint32),
        spheroidal=np.zeros((S, S), np.float32),
        aterms=np.zeros((ntimeslots, nstations, S, S, 4), np.complex64),
        metadata=np.zeros(nsg, METADATA_DTYPE),
    )
    ref().ref_init_dataset(grid_size, subgrid_size, nstations, nchannels, ntimeslots, ntimesteps,
                           *[_p(d[k]) for k in ("uvw", "frequencies", "wavenumbers", "vis", "baselines",
                                                "spheroidal", "aterms", "metadata")])
    return d


def ref_subgrids(n_subgrids, subgrid_size):
    out = np.zeros((n_subgrids, 4, subgrid_size, subgrid_size), np.complex64)
    ref().ref_init_subgrids(n_subgrids, subgrid_size, _p(out))
    return out


def _ref_run(fn, cfg, d, subgrids, niterations=1):
    G, S, ns, C, nts, T = cfg
    return fn(G, S, ns, C, nts, T, niterations, *[_p(d[k]) for k in ("uvw", "frequencies", "wavenumbers", "vis", "baselines",
                                                                        "spheroidal", "aterms")],
              _p(subgrids), _p(d["metadata"]))


def ref_cpu_gridding(cfg, d, niterations=1):
    """Runs gridding_benchmark_launcher<cpu>::launch; returns (subgrids, mean compute us)."""
    G, S, ns, C, nts, T = cfg
    nsg = ns * (ns - 1) // 2 * nts
    sub = np.zeros((nsg, 4, S, S), np.complex64)
    us = _ref_run(ref().ref_cpu_gridding, cfg, d, sub, niterations)
    return sub, us


def ref_cpu_degridding(cfg, d, subgrids, niterations=1):
    """Runs degridding_benchmark_launcher<cpu>::launch on `subgrids`; returns (vis, mean compute us)."""
    dd = dict(d)
    dd["vis"] = np.zeros_like(d["vis"])
    sub = np.ascontiguousarray(subgrids, np.complex64)
    us = _ref_run(ref().ref_cpu_degridding, cfg, dd, sub, niterations)
    return dd["vis"], us
