"""The drop-in launcher pair on the GPU: gridding_benchmark_launcher<gpu>::launch
and degridding_benchmark_launcher<gpu>::launch (gridding/src/gridding_benchmark.cu:248-361,
gridding/src/degridding_benchmark.cu:205-318), reached through the Python
mirror and the C ABI's idg_gridding_launch / idg_degridding_launch.

On the reference's own inputs and random plans (the three golden cases, made
by the reference's generators; image_size 0.1 as the reference hard-codes):
- the subgrids the launcher copies out are within 1e-5 (relative RMS) of the
  FP64 oracle and within 5e-4 of the reference's FP32 CPU output;
- the visibilities are checked the same way, with the reference CPU's A-term
  convention (IDG_FLAG_DEGRID_ATERM_REFCPU);
- benchmark_result follows gridding_benchmark.cu:322-358: times in
  microseconds per iteration, bandwidths in bytes per microsecond over the
  whole niterations loop (so bandwidth x time x niterations = the bytes one
  iteration copies), and niterations repeats leave the outputs unchanged.
The CLI (python -m idg_gb300) on a hardware_types: [gpu] YAML writes the
12-column ';' CSV with measured values.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import idg_gb300._lib as L
from conftest import PKG, check_rel, golden_cases, load_golden, rel_rms

pytestmark = pytest.mark.gpu

TOL = 1e-5
VARIANTS = [L.VARIANT_PLAIN, L.VARIANT_BATCHED]


def _cfg(d, niterations, variant):
    from idg_gb300 import launcher

    G, S, ns, C, nts, T = d["cfg"]
    return launcher.configuration(htype=launcher.hardware_type.gpu, niterations=niterations, grid_size=G,
                                  subgrid_size=S, nstations=ns, nchannels=C, ntimeslots=nts,
                                  ntimesteps_per_subgrid=T, degrid_aterm_refcpu=True, variant=variant)


def _in_bytes(d, gridding):
    """Bytes one iteration copies in (uvw, wavenumbers, spheroidal, A-terms,
    plan, and the visibilities or, for the degridder, the subgrids)."""
    n = d["uvw"].nbytes + d["wavenumbers"].nbytes + d["spheroidal"].nbytes + d["aterms"].nbytes
    n += d["metadata"].shape[0] * 36
    return n + (d["vis"].nbytes if gridding else d["degridder_in"].nbytes)


def _check_result(r, niterations, in_bytes, out_bytes):
    for f in ("in_transfer_time", "out_transfer_time", "in_bandwidth", "out_bandwidth", "compute_time"):
        assert getattr(r, f) > 0, f
    # bandwidth (bytes/us, whole loop) x time (us per iteration) x niterations = bytes per iteration
    assert r.in_bandwidth * r.in_transfer_time * niterations == pytest.approx(in_bytes, rel=1e-6)
    assert r.out_bandwidth * r.out_transfer_time * niterations == pytest.approx(out_bytes, rel=1e-6)


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.rsplit("/", 1)[-1])
@pytest.mark.parametrize("variant", VARIANTS)
def test_launcher_pair_on_reference_inputs(oracle_mod, idg, path, variant):
    from idg_gb300 import launcher

    d = load_golden(path)
    G, S, ns, C, nts, T = d["cfg"]
    nsg = d["metadata"].shape[0]
    prm = oracle_mod.params(G, S, C, ns, nsg, 0.1)
    want_sub = oracle_mod.gridder(prm, d["uvw"], d["wavenumbers"], d["vis"], d["spheroidal"], d["aterms"],
                                  d["metadata"])
    want_vis = oracle_mod.degridder(prm, d["uvw"], d["wavenumbers"], d["degridder_in"], d["spheroidal"],
                                    d["aterms"], d["metadata"], d["vis"].shape[0], aterm_mode=oracle_mod.ATERM_REFCPU)
    runs = {}
    for niter in (1, 3):
        cfg = _cfg(d, niter, variant)
        sub = np.full((nsg, 4, S, S), np.nan, np.complex64)
        r = launcher.gridding_benchmark_launcher.launch(cfg, d["uvw"], d["vis"], d["baselines"], d["aterms"],
                                                       d["frequencies"], d["wavenumbers"], d["spheroidal"], sub,
                                                       d["metadata"])
        check_rel(f"launcher gridding {os.path.basename(path)} v{variant} x{niter}", sub, want_sub, TOL)
        assert rel_rms(sub, d["gridder_out"]) < 5e-4
        _check_result(r, niter, _in_bytes(d, True), sub.nbytes)

        vis = np.full_like(d["vis"], np.nan)
        r = launcher.degridding_benchmark_launcher.launch(cfg, d["uvw"], vis, d["baselines"], d["aterms"],
                                                         d["frequencies"], d["wavenumbers"], d["spheroidal"],
                                                         d["degridder_in"], d["metadata"])
        check_rel(f"launcher degridding {os.path.basename(path)} v{variant} x{niter}", vis, want_vis, TOL)
        assert rel_rms(vis, d["degridder_out"]) < 5e-4
        _check_result(r, niter, _in_bytes(d, False), vis.nbytes)
        runs[niter] = (sub, vis)
    # repeating the kernels niterations times changes nothing
    assert np.array_equal(runs[1][0], runs[3][0])
    assert np.array_equal(runs[1][1], runs[3][1])


def test_cli_gpu_configuration_writes_the_csv(idg, tmp_path):
    """gridding-benchmarks <config.yaml> <output.csv> (gridding/src/main.cpp:139-163)
    with the GPU hardware type: the table and the 12-column CSV, one row per
    (operation, hardware) pair, with measured times."""
    yaml = tmp_path / "gpu.yaml"
    yaml.write_text("grid_size: 1024\noperation_types: [gridding, degridding]\nniterations: 2\nnstations: 4\n"
                    "ntimeslots: 2\nntimesteps_per_subgrid: 64\nnchannels: 16\nsubgrid_size: 32\n"
                    "hardware_types: [gpu]\n")
    env = {**os.environ, "PYTHONPATH": PKG + os.pathsep + os.environ.get("PYTHONPATH", "")}
    r = subprocess.run([sys.executable, "-m", "idg_gb300", str(yaml), "result.csv"], cwd=tmp_path, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = (tmp_path / "result.csv").read_text().split("\n")
    assert lines[-1] == ""
    rows = [ln.split(";") for ln in lines[:-1]]
    assert len(rows) == 3
    for row in rows:
        assert len(row) == 13 and row[-1] == ""  # 12 fields, each followed by ';'
    assert [row[1] for row in rows[1:]] == ["gridding", "degridding"]
    for row in rows[1:]:
        assert row[2] == "2" and row[3] == "1024" and row[4] == "32"
        nums = [float(x) for x in row[7:12]]  # in/out transfer time, compute time, in/out bandwidth
        assert all(x > 0 for x in nums), row
