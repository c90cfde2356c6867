"""The reference-side binding (integration/gpu_launchers.cpp) compiles against
the reference's own headers and links with the reference's CPU sources and
libidg_gb300.so into a working gridding-benchmarks program.  CPU only: the
program is run on a CPU configuration (the GPU specialisation is linked,
not executed).  Skipped where the reference sources are not present."""
import os
import subprocess

import pytest

from conftest import PKG, ROOT
from oracle import REFERENCE_DIR as REFERENCE

MAIN = r"""
#include <cstdio>
#include "gridding_benchmark.h"
#include "degridding_benchmark.h"
using namespace gridding_benchmark;
int main() {
    configuration c{};
    c.htype = benchmarks_common::hardware_type::cpu;
    c.operation = operation_type::gridding;
    c.niterations = 1; c.grid_size = 256; c.subgrid_size = 16; c.nstations = 3;
    c.nchannels = 4; c.ntimeslots = 1; c.ntimesteps_per_subgrid = 8;
    benchmark_result r = launch_gridding(c);
    benchmark_result d = launch_degridding(c);
    // the GPU specialisations are present in the binary
    auto *g = &gridding_benchmark_launcher<benchmarks_common::hardware_type::gpu>::launch;
    auto *h = &degridding_benchmark_launcher<benchmarks_common::hardware_type::gpu>::launch;
    std::printf("ok %d %d %d\n", r.compute_time > 0, d.compute_time > 0, g != nullptr && h != nullptr);
    return 0;
}
"""


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(REFERENCE), reason="reference sources not present")
def test_shim_links_into_reference_program(idg, tmp_path):
    from idg_gb300 import _lib

    lib = _lib.lib_path()
    g = os.path.join(REFERENCE, "gridding")
    srcs = [os.path.join(g, "src", f) for f in ("gridding_benchmark.cpp", "degridding_benchmark.cpp",
                                                 "gridding_initialization.cpp")]
    main = tmp_path / "main.cpp"
    main.write_text(MAIN)
    exe = tmp_path / "gridding-benchmarks"
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DENABLE_OMP", "-DENABLE_CPU=1", "-DENABLE_GPU=1", "-w",
           "-I", os.path.join(g, "inc"), "-I", os.path.join(REFERENCE, "benchmarks-common", "inc"),
           "-I", os.path.join(ROOT, "include"),
           str(main), os.path.join(PKG, "integration", "gpu_launchers.cpp"), *srcs,
           lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "ok 1 1 1"
