"""The C ABI on the host: the library builds, loads and exports every entry
point include/idg_gb300.h declares; argument checks fail with the documented
codes before any device work; the reference-compatible generator reproduces
the reference's inputs value for value.  CPU only (no kernel is launched)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden

HEADER = os.path.join(ROOT, "include", "idg_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"IDG_API\s+[\w\s\*]+?\b(idg_\w+)\s*\(", text)))


def test_header_and_binding_agree(idg):
    from idg_gb300 import _lib

    assert set(declared_symbols()) == set(_lib.exported_symbols())


def test_header_constants_match_the_binding(idg):
    """Every status code, flag, variant and job kind of the header has the same
    value in the Python binding (IDG_VARIANT_* are VARIANT_* there)."""
    from idg_gb300 import _lib

    text = open(HEADER).read()
    consts = {m[0]: int(m[1], 0) for m in re.findall(r"#define\s+(IDG_(?:FLAG|VARIANT|JOB)_\w+)\s+(0x[0-9a-fA-F]+|\d+)u?",
                                                     text)}
    consts.update({m[0]: int(m[1]) for m in re.findall(r"\b(IDG_(?:OK|ERR_\w+))\s*=\s*(\d+)", text)})
    assert len(consts) >= 15
    for name, value in consts.items():
        py = name.replace("IDG_VARIANT_", "VARIANT_")
        assert getattr(_lib, py) == value, name


def test_library_exports_every_declared_symbol(idg):
    lib = idg.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.idg_abi_version() == 4


def test_library_is_in_tree(idg):
    from idg_gb300 import _lib

    assert os.path.realpath(_lib.lib_path()).startswith(os.path.realpath(ROOT))


def test_argument_errors_before_device_work(idg):
    from idg_gb300 import _lib

    lib = idg.load()
    p = _lib.IdgParams(1024, 32, 16, 4, 1, 1, 0.1, 0.0, 0, 0)
    # NULL params
    assert lib.idg_gridder(None, 0, 1, None, None, 1, None, None, None, None, None, None, None) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "params" in _lib.last_error()
    # odd subgrid size
    bad = _lib.IdgParams(1024, 33, 16, 4, 1, 1, 0.1, 0.0, 0, 0)
    assert lib.idg_gridder(ctypes.byref(bad), 0, 1, None, None, 1, None, None, None, None, None, None, None) == _lib.IDG_ERR_UNSUPPORTED
    # too many channels
    bad = _lib.IdgParams(1024, 32, 2000, 4, 1, 1, 0.1, 0.0, 0, 0)
    assert lib.idg_degridder(ctypes.byref(bad), 0, 1, None, None, 1, None, None, None, None, None, None, None) == _lib.IDG_ERR_UNSUPPORTED
    # unknown variant
    assert lib.idg_gridder(ctypes.byref(p), 7, 1, None, None, 1, None, None, None, None, None, None, None) == _lib.IDG_ERR_INVALID_ARGUMENT
    # NULL device pointers with work to do
    assert lib.idg_gridder(ctypes.byref(p), 0, 1, None, None, 1, None, None, None, None, None, None, None) == _lib.IDG_ERR_INVALID_ARGUMENT
    # empty plan is a no-op
    assert lib.idg_gridder(ctypes.byref(p), 0, 0, None, None, 0, None, None, None, None, None, None, None) == _lib.IDG_OK
    # FFT sizes
    p40 = _lib.IdgParams(1024, 40, 16, 4, 1, 1, 0.1, 0.0, 0, 0)
    assert lib.idg_subgrid_fft(ctypes.byref(p40), 1, 1, None, None, None) == _lib.IDG_ERR_UNSUPPORTED
    assert lib.idg_subgrid_fft(ctypes.byref(p), 1, 0, None, None, None) == _lib.IDG_ERR_INVALID_ARGUMENT
    # splitter + backward FFT in one pass: FFT sizes, counts and pointers checked first
    assert lib.idg_split_subgrid_fft(ctypes.byref(p40), 1, None, None, None, None, None) == _lib.IDG_ERR_UNSUPPORTED
    assert lib.idg_split_subgrid_fft(ctypes.byref(p), -1, None, None, None, None, None) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert lib.idg_split_subgrid_fft(ctypes.byref(p), 1, None, None, None, None, None) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert lib.idg_split_subgrid_fft(ctypes.byref(p), 0, None, None, None, None, None) == _lib.IDG_OK
    # launcher config
    cfg = _lib.IdgLaunchConfig(0, 1024, 32, 4, 16, 1, 32, 0.1, 0.0, 0, 0)
    r = _lib.IdgBenchmarkResult()
    assert lib.idg_gridding_launch(ctypes.byref(cfg), None, None, None, None, None, None, None, None, None, ctypes.byref(r)) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "niterations" in _lib.last_error()


def test_imaging_cycles_argument_errors_before_device_work(idg):
    """idg_imaging_cycles checks its cycles on the host, before any CUDA call:
    counts, NULL arrays and rows (reported with the cycle's index), and host
    memory that a later cycle would read before an earlier one writes it."""
    from idg_gb300 import _lib

    lib = idg.load()
    p = _lib.IdgParams(1024, 32, 4, 4, 1, 1, 0.1, 0.0, 0, 0)
    C, rows = 4, 16
    md = np.zeros(2, _lib.METADATA_DTYPE)
    md["nr_timesteps"] = 8
    md["time_offset"] = [0, 8]
    uvw = np.zeros((rows, 3), np.float32)
    k = np.zeros(C, np.float32)
    taper = np.zeros((32, 32), np.float32)
    at = np.zeros((1, 4, 32, 32, 4), np.complex64)
    bufs = [np.zeros((rows, C, 4), np.complex64) for _ in range(4)]

    def io(vin, vout, nr_rows=rows, m=md):
        return _lib.IdgCycleIo(m.shape[0], m.ctypes.data, nr_rows, uvw.ctypes.data, vin.ctypes.data,
                               vout.ctypes.data, None, None)

    def run(*cycles, n=None):
        arr = (_lib.IdgCycleIo * max(1, len(cycles)))(*cycles)
        return lib.idg_imaging_cycles(ctypes.byref(p), 0, len(cycles) if n is None else n, arr, k.ctypes.data,
                                      taper.ctypes.data, at.ctypes.data, 0)

    assert lib.idg_imaging_cycles(ctypes.byref(p), 0, 1, None, None, None, None, 0) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert run(io(bufs[0], bufs[1]), n=0) == _lib.IDG_ERR_INVALID_ARGUMENT
    # more cycles than one call takes (checked before the array is read)
    assert run(io(bufs[0], bufs[1]), n=4097) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "nr_cycles outside [1, 4096]" in _lib.last_error()
    # cycle 1 names rows past its nr_rows
    assert run(io(bufs[0], bufs[1]), io(bufs[0], bufs[1], nr_rows=12)) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "cycle 1: plan entry 1" in _lib.last_error()
    # cycle 1 reads what cycle 0 writes (its output fed back as input)
    assert run(io(bufs[0], bufs[1]), io(bufs[1], bufs[2])) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "cycle 1 reads host memory that cycle 0 writes" in _lib.last_error()
    # ... or a part of it
    half = bufs[1][rows // 2:]
    assert run(io(bufs[0], bufs[1]), io(bufs[2], bufs[3]), io(half, bufs[3])) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "cycle 2 reads host memory that cycle 0 writes" in _lib.last_error()
    # a NULL array in a later cycle
    bad = io(bufs[0], bufs[1])
    bad.uvw = None
    assert run(io(bufs[0], bufs[1]), bad) == _lib.IDG_ERR_INVALID_ARGUMENT
    assert "cycle 1: NULL host array" in _lib.last_error()


def test_python_wrapper_raises(idg):
    from idg_gb300 import _lib

    with pytest.raises(_lib.IdgError) as e:
        _lib.call("idg_subgrid_fft", None, 1, 1, None, None, None)
    assert e.value.code == _lib.IDG_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.rsplit("/", 1)[-1])
def test_reference_dataset_matches_reference(idg, path):
    from idg_gb300 import launcher as L

    d = load_golden(path)
    G, S, ns, C, nts, T = d["cfg"]
    cfg = L.configuration(grid_size=G, subgrid_size=S, nstations=ns, nchannels=C, ntimeslots=nts,
                          ntimesteps_per_subgrid=T)
    got = L.reference_dataset(cfg)
    for k_got, k_ref in [("uvw", "uvw"), ("frequencies", "frequencies"), ("wavenumbers", "wavenumbers"),
                         ("visibilities", "vis"), ("baselines", "baselines"), ("spheroidal", "spheroidal"),
                         ("aterms", "aterms")]:
        a, b = getattr(got, k_got), d[k_ref]
        assert a.shape == b.shape, k_got
        assert np.array_equal(a.view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), k_got
    assert np.array_equal(got.metadata.view(np.uint8), d["metadata"].view(np.uint8))
    # the reference's initialize_subgrids pattern (used as degridder input)
    assert np.array_equal(L.reference_subgrids(d["degridder_in"].shape[0], S).view(np.uint32),
                          d["degridder_in"].view(np.uint32))
