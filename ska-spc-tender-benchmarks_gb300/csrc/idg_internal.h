// idg_internal.h -- launch functions shared between the kernel files and the C ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace idg {

struct KernelArgs;

// IDG_VARIANT_PLAIN: one CTA per subgrid (idg_gridder.cu / idg_degridder.cu).
// IDG_VARIANT_BATCHED: persistent packed-FP32x2 kernels (idg_*_fast.cu); need a.work_counter.
cudaError_t launch_gridder(const KernelArgs &a, int variant, int max_nc, cudaStream_t stream);
cudaError_t launch_degridder(const KernelArgs &a, int variant, int max_nc, cudaStream_t stream);
// shape: index into the batched gridder's launch shapes (see gridder_fast_shapes()).
cudaError_t launch_gridder_fast(const KernelArgs &a, cudaStream_t stream, int shape);
int gridder_fast_shapes();
// Loads the kernels of every batched gridder shape into the current device's
// context without launching them.
cudaError_t load_gridder_fast();
// The shape the batched gridder uses on the current device for subgrid size S.
int batched_gridder_shape(int S);
void set_batched_gridder_shape(int S, int shape);
cudaError_t launch_degridder_fast(const KernelArgs &a, cudaStream_t stream, int shape);
int degridder_fast_shapes();
// Channel-pair-packed batched degridder (idg_degridder_cp.cu), shapes 0..degridder_cp_shapes()-1.
cudaError_t launch_degridder_cp(const KernelArgs &a, cudaStream_t stream, int shape);
int degridder_cp_shapes();
int batched_degridder_shape(int S);
void set_batched_degridder_shape(int S, int shape);

bool fft_size_supported(int S);
cudaError_t launch_subgrid_fft(float2 *data, int64_t nr_subgrids, int S, int direction, const float *taper,
                               cudaStream_t stream);
// The degridding step's splitter and backward subgrid FFT in one pass (same
// result as launch_splitter followed by launch_subgrid_fft with direction -1).
cudaError_t launch_split_fft(const struct idg_metadata *md, int64_t nr_subgrids, int S, int G, int W,
                             const float2 *grid, float2 *subgrids, const float *taper, cudaStream_t stream);

bool grid_fft_size_supported(int G);
cudaError_t launch_grid_fft(float2 *grid, int G, int planes, int direction, const float *correction,
                            unsigned *status, bool test_lost_copy, cudaStream_t stream);

cudaError_t launch_adder(const struct idg_metadata *md, int64_t nr_subgrids, int S, int G, int W,
                         const float2 *subgrids, float2 *grid, cudaStream_t stream);
cudaError_t launch_splitter(const struct idg_metadata *md, int64_t nr_subgrids, int S, int G, int W,
                            const float2 *grid, float2 *subgrids, cudaStream_t stream);

cudaError_t measure_fp32_peak(double *flops);

} // namespace idg
