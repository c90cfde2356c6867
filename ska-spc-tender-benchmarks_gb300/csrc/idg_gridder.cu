// idg_gridder.cu -- gridder kernels.
//
// Computes, for every subgrid s of the plan and every pixel (x, y),
//   P[pol] = sum_{t, c} V[t][c][pol] * exp(i * 2*pi * tau(x, y, t, c))
//   subgrid[s][pol][y][x] = taper(y, x) * (A1^H P A2)[pol]
// which is the reference's gridder (gridding/src/gridding_benchmark.cpp:56-166,
// kernel_gridder_v7 at gridding/src/gridding_benchmark.cu:19-246) with the
// phase carried as described in idg_device.cuh.
//
// Work decomposition (plain variant): one CTA of 256 threads per subgrid; each
// thread owns PPT pixels (strided by 256 so stores coalesce) and keeps their
// four complex accumulators in registers for the whole time/channel sweep.
// Visibilities of a time tile and the tile's FP64-derived phase coefficients
// are staged in shared memory and read as warp-wide broadcasts.  Per
// pixel-visibility the inner loop issues 1 FFMA (phase), 3 FADD (reduction to
// [-1/2, 1/2] turns), the sincos and 16 FFMA (4 complex MACs).
#include "idg_device.cuh"
#include "idg_internal.h"

namespace idg {

namespace {

constexpr int kThreads = 256;
constexpr int kPPT = 4;                 // pixels per thread per pass
constexpr int kVisTileBudget = 1024;    // visibilities per staged tile (32 KiB)
constexpr int kMaxTileTimesteps = 128;

// Timesteps per staged tile: tt * nc <= kVisTileBudget for every nc >= 1, so
// one fixed shared-memory carve (see smem layout below) fits any subgrid.
__host__ __device__ inline int tile_timesteps(int nc) {
    int tt = kVisTileBudget / (nc > 0 ? nc : 1);
    if (tt > kMaxTileTimesteps) tt = kMaxTileTimesteps;
    if (tt < 1) tt = 1;
    return tt;
}

// Shared-memory layout (float4 units): [0, 2*kMaxTileTimesteps) phase
// coefficients, then 2*kVisTileBudget visibility slots, then max_nc floats of
// channel offsets.
constexpr int kCoefSlots = 2 * kMaxTileTimesteps;
constexpr int kVisSlots = 2 * kVisTileBudget;

// One pass over PPT pixels per thread for subgrid `s`, all timesteps.
__device__ __forceinline__ void grid_subgrid(const KernelArgs &a, const SubgridInfo &si, int s, float4 *coef_s,
                                             float4 *vis_s, float *kappa_s) {
    const int tid = threadIdx.x;
    const int S = a.S, S2 = S * S;
    const int nc = si.c1 - si.c0;
    const int TT = tile_timesteps(nc);

    // channel offsets relative to the subgrid's first channel (exact in FP64, rounded once)
    __syncthreads();
    for (int c = tid; c < nc; c += kThreads)
        kappa_s[c] = (float)((double)a.wavenumbers[si.c0 + c] - (double)a.wavenumbers[si.c0]);

    for (int pbase = 0; pbase < S2; pbase += kThreads * kPPT) {
        float hx[kPPT], hy[kPPT], nn[kPPT];
        cf acc[kPPT][4];
#pragma unroll
        for (int k = 0; k < kPPT; ++k) {
            const int q = pbase + tid + k * kThreads;
            const float3 g = pixel_geometry(q < S2 ? q : 0, S, a.image_size);
            hx[k] = g.x;
            hy[k] = g.y;
            nn[k] = g.z;
#pragma unroll
            for (int p = 0; p < 4; ++p) acc[k][p] = {0.f, 0.f};
        }

        for (int t0 = 0; t0 < si.T; t0 += TT) {
            const int tt = min(TT, si.T - t0);
            __syncthreads();
            for (int t = tid; t < tt; t += kThreads) time_coefficients(a, si, t0 + t, coef_s + 2 * t);
            {
                const int per_row = nc * 2; // float4 per row
                const float4 *src = a.vis + ((int64_t)si.row0 + t0) * a.C * 2 + (int64_t)si.c0 * 2;
                for (int i = tid; i < tt * per_row; i += kThreads) {
                    const int r = i / per_row, e = i - r * per_row;
                    vis_s[i] = src[(int64_t)r * a.C * 2 + e];
                }
            }
            __syncthreads();

            for (int t = 0; t < tt; ++t) {
                const float4 c0 = coef_s[2 * t], c1 = coef_s[2 * t + 1];
                float tau0[kPPT], Q[kPPT];
#pragma unroll
                for (int k = 0; k < kPPT; ++k) {
                    tau0[k] = frac_turns(fmaf(c0.x, hx[k], fmaf(c0.y, hy[k], c0.z * nn[k])));
                    Q[k] = fmaf(c0.w, hx[k], fmaf(c1.x, hy[k], c1.y * nn[k]));
                }
                const float4 *vrow = vis_s + t * nc * 2;
#pragma unroll 2
                for (int c = 0; c < nc; ++c) {
                    const float kap = kappa_s[c];
                    const float4 va = vrow[2 * c], vb = vrow[2 * c + 1];
#pragma unroll
                    for (int k = 0; k < kPPT; ++k) {
                        const float r = frac_turns(fmaf(kap, Q[k], tau0[k]));
                        float sn, cs;
                        sincos_turns(r, &sn, &cs);
                        cmac(acc[k][0], {va.x, va.y}, cs, sn);
                        cmac(acc[k][1], {va.z, va.w}, cs, sn);
                        cmac(acc[k][2], {vb.x, vb.y}, cs, sn);
                        cmac(acc[k][3], {vb.z, vb.w}, cs, sn);
                    }
                }
            }
        }

        // epilogue: A-terms, taper, store
        const size_t jones_stride = (size_t)S2 * 2; // float4 per station image
        const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
        const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;
#pragma unroll
        for (int k = 0; k < kPPT; ++k) {
            const int q = pbase + tid + k * kThreads;
            if (q >= S2) continue;
            cf j1[4], j2[4];
            load_jones(a1 + 2 * q, j1);
            load_jones(a2 + 2 * q, j2);
            aterm_gridder(acc[k], j1, j2);
            const float sph = (a.flags & IDG_FLAG_NO_TAPER) ? 1.f : a.taper[q];
#pragma unroll
            for (int p = 0; p < 4; ++p)
                a.subgrids[((size_t)s * 4 + p) * S2 + q] = make_float2(acc[k][p].re * sph, acc[k][p].im * sph);
        }
    }
}

__device__ __forceinline__ void zero_subgrid(const KernelArgs &a, int s) {
    const int S2 = a.S * a.S;
    for (int i = threadIdx.x; i < 4 * S2; i += kThreads) a.subgrids[(size_t)s * 4 * S2 + i] = make_float2(0.f, 0.f);
}

__global__ void __launch_bounds__(kThreads) gridder_plain_kernel(KernelArgs a) {
    extern __shared__ float4 smem[];
    const int s = blockIdx.x;
    const SubgridInfo si = load_subgrid(a, s);
    if (!si.ok) {
        if (threadIdx.x == 0) flag_status(a.status, kStatusBadPlan);
        zero_subgrid(a, s);
        return;
    }
    float4 *coef_s = smem;
    float4 *vis_s = coef_s + kCoefSlots;
    float *kappa_s = (float *)(vis_s + kVisSlots);
    grid_subgrid(a, si, s, coef_s, vis_s, kappa_s);
}

size_t smem_bytes_for(int max_nc) { return (size_t)(kCoefSlots + kVisSlots) * 16 + (size_t)max_nc * 4 + 16; }

} // namespace

cudaError_t launch_gridder(const KernelArgs &a, int variant, int max_nc, cudaStream_t stream) {
    const size_t smem = smem_bytes_for(max_nc);
    if (variant == IDG_VARIANT_PLAIN) {
        cudaError_t e = cudaFuncSetAttribute(gridder_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        gridder_plain_kernel<<<(unsigned)a.nr_subgrids, kThreads, smem, stream>>>(a);
        return cudaGetLastError();
    }
    return launch_gridder_fast(a, stream, batched_gridder_shape(a.S));
}

} // namespace idg
