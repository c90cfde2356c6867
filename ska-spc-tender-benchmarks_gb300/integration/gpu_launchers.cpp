// gpu_launchers.cpp -- the reference benchmark's GPU launcher specialisations,
// implemented on top of libidg_gb300.so.
//
// Drop-in replacement for gridding/src/gridding_benchmark.cu and
// gridding/src/degridding_benchmark.cu of ska-spc-tender-benchmarks: it
// defines
//   gridding_benchmark_launcher<hardware_type::gpu>::launch   (gridding_benchmark.h:10-21)
//   degridding_benchmark_launcher<hardware_type::gpu>::launch (degridding_benchmark.h:18-28)
// with the same arguments and the same benchmark_result (common_gridding.h:5-12),
// so the reference's launch_gridding / launch_degridding / main.cpp run
// unchanged on the GB300 kernels.  It is plain C++ (no CUDA compiler needed)
// and is compiled against the reference's headers and include/idg_gb300.h.
//
// Behaviour kept from the reference: image_size 0.1 and w_step 0 (the values
// its GPU launchers hard-code, gridding_benchmark.cu:315-316), one timed
// copy-in / compute / copy-out phase per call with `niterations` repetitions,
// and exit(code) on any failure (util.cuh:9-16).  Differences, on purpose:
// the gridder's subgrids are copied device-to-host into `subgrids` (the
// reference copies them host-to-device, gridding_benchmark.cu:345), and the
// degridder copies `subgrids` in and `visibilities` out (the reference does
// neither, degridding_benchmark.cu:255-303).
#include <cstdio>
#include <cstdlib>

#include "degridding_benchmark.h"
#include "gridding_benchmark.h"
#include "idg_gb300.h"

namespace gridding_benchmark {

namespace {

idg_launch_config to_idg(const configuration &c, bool degridding) {
    idg_launch_config k{};
    k.niterations = (int64_t)c.niterations;
    k.grid_size = (int64_t)c.grid_size;
    k.subgrid_size = (int64_t)c.subgrid_size;
    k.nstations = (int64_t)c.nstations;
    k.nchannels = (int64_t)c.nchannels;
    k.ntimeslots = (int64_t)c.ntimeslots;
    k.ntimesteps_per_subgrid = (int64_t)c.ntimesteps_per_subgrid;
    k.image_size = 0.1F;
    k.w_step = 0.F;
    // the reference's degridder on the CPU applies A1^H P A2 (degridding_benchmark.cpp:113)
    k.flags = degridding ? IDG_FLAG_DEGRID_ATERM_REFCPU : 0u;
    k.variant = IDG_VARIANT_BATCHED;
    return k;
}

benchmark_result to_reference(const idg_benchmark_result &r) {
    benchmark_result out;
    out.in_transfer_time = r.in_transfer_time;
    out.out_transfer_time = r.out_transfer_time;
    out.in_bandwidth = r.in_bandwidth;
    out.out_bandwidth = r.out_bandwidth;
    out.compute_time = r.compute_time;
    return out;
}

void check(int rc) {
    if (rc != IDG_OK) {
        std::fprintf(stderr, "GPUassert: %s\n", idg_last_error());
        std::exit(rc);
    }
}

} // namespace

template <>
benchmark_result gridding_benchmark_launcher<benchmarks_common::hardware_type::gpu>::launch(
    const configuration &configuration, Array2D<UVWCoordinate<float>> &uvw,
    Array3D<Visibility<std::complex<float>>> &visibilities, Array1D<Baseline> &baselines,
    Array4D<Matrix2x2<std::complex<float>>> &aterms, Array1D<float> &frequencies, Array1D<float> &wavenumbers,
    Array2D<float> &spheroidal, Array4D<std::complex<float>> &subgrids, Array1D<Metadata> &metadata) {
    static_assert(sizeof(Metadata) == sizeof(idg_metadata), "Metadata layout");
    const idg_launch_config cfg = to_idg(configuration, false);
    idg_benchmark_result r{};
    check(idg_gridding_launch(&cfg, reinterpret_cast<const float *>(uvw.data()), visibilities.data(),
                              reinterpret_cast<const uint32_t *>(baselines.data()), aterms.data(), frequencies.data(),
                              wavenumbers.data(), spheroidal.data(), subgrids.data(),
                              reinterpret_cast<const idg_metadata *>(metadata.data()), &r));
    return to_reference(r);
}

template <>
benchmark_result degridding_benchmark_launcher<benchmarks_common::hardware_type::gpu>::launch(
    const configuration &configuration, Array2D<UVWCoordinate<float>> &uvw,
    Array3D<Visibility<std::complex<float>>> &visibilities, Array1D<Baseline> &baselines,
    Array4D<Matrix2x2<std::complex<float>>> &aterms, Array1D<float> &frequencies, Array1D<float> &wavenumbers,
    Array2D<float> &spheroidal, Array4D<std::complex<float>> &subgrids, Array1D<Metadata> &metadata) {
    const idg_launch_config cfg = to_idg(configuration, true);
    idg_benchmark_result r{};
    check(idg_degridding_launch(&cfg, reinterpret_cast<const float *>(uvw.data()), visibilities.data(),
                                reinterpret_cast<const uint32_t *>(baselines.data()), aterms.data(),
                                frequencies.data(), wavenumbers.data(), spheroidal.data(), subgrids.data(),
                                reinterpret_cast<const idg_metadata *>(metadata.data()), &r));
    return to_reference(r);
}

} // namespace gridding_benchmark
