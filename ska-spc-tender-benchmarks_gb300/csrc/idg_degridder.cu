// idg_degridder.cu -- degridder kernels.
//
// For every subgrid s and every (t, c) it covers,
//   V[t][c][pol] = sum_{y,x} P'[pol](x, y) * exp(-i * 2*pi * tau(x, y, t, c))
// with P' = A(taper * subgrid) and A the adjoint A-term A1 P A2^H (the
// reference's GPU convention, common_gridding.cuh:82-94) or, with
// IDG_FLAG_DEGRID_ATERM_REFCPU, the reference CPU's A1^H P A2
// (degridding_benchmark.cpp:113).  The w-offset follows the CPU launcher
// (2*pi*w_step*(z+1/2), degridding_benchmark.cpp:129), not the GPU kernel's
// (z+1/2)*2*pi (degridding_benchmark.cu:33).
//
// Work decomposition: one CTA of 256 threads per subgrid (plain) or per
// pulled work item (persistent).  The CTA stages up to 1024 prepared pixels
// (P' plus {hx, hy, n}) in shared memory.  A warp works on 8 visibility groups
// at once, each group = one timestep x kCB channels, shared by 4 lanes that
// split the pixels four ways; every lane keeps its group's kCB x 4 complex
// partial sums in registers and the 4 lanes are combined with warp shuffles.
#include "idg_device.cuh"
#include "idg_internal.h"

namespace idg {

namespace {

constexpr int kThreads = 256;
constexpr int kCB = 8;              // channels per visibility group
constexpr int kLanesPerGroup = 4;   // lanes sharing one group's pixels
constexpr int kPixBatch = 1024;     // pixels staged per pass
constexpr int kTimeTile = 64;       // timesteps whose coefficients are staged per pass

__device__ __forceinline__ void degrid_subgrid(const KernelArgs &a, const SubgridInfo &si, int s, float4 *pix_s,
                                               float4 *geo_s, float4 *coef_s, float *kappa_s) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int S = a.S, S2 = S * S;
    const int nc = si.c1 - si.c0;
    const int ncb = (nc + kCB - 1) / kCB;
    const int g_in_warp = lane / kLanesPerGroup; // 0..7
    const int part = lane % kLanesPerGroup;      // 0..3
    const bool refcpu = (a.flags & IDG_FLAG_DEGRID_ATERM_REFCPU) != 0;
    const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;

    __syncthreads();
    for (int c = tid; c < nc; c += kThreads)
        kappa_s[c] = (float)((double)a.wavenumbers[si.c0 + c] - (double)a.wavenumbers[si.c0]);

    const size_t jones_stride = (size_t)S2 * 2;
    const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
    const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;

    for (int pbase = 0; pbase < S2; pbase += kPixBatch) {
        const int np = min(kPixBatch, S2 - pbase);
        __syncthreads();
        for (int i = tid; i < np; i += kThreads) {
            const int q = pbase + i;
            cf p[4];
            const float sph = taper ? a.taper[q] : 1.f;
#pragma unroll
            for (int pol = 0; pol < 4; ++pol) {
                const float2 v = a.subgrids[((size_t)s * 4 + pol) * S2 + q];
                p[pol] = {sph * v.x, sph * v.y};
            }
            cf j1[4], j2[4];
            load_jones(a1 + 2 * q, j1);
            load_jones(a2 + 2 * q, j2);
            if (refcpu)
                aterm_gridder(p, j1, j2);
            else
                aterm_adjoint(p, j1, j2);
            pix_s[2 * i] = make_float4(p[0].re, p[0].im, p[1].re, p[1].im);
            pix_s[2 * i + 1] = make_float4(p[2].re, p[2].im, p[3].re, p[3].im);
            const float3 g = pixel_geometry(q, S, a.image_size);
            geo_s[i] = make_float4(g.x, g.y, g.z, 0.f);
        }

        for (int t0 = 0; t0 < si.T; t0 += kTimeTile) {
            const int tt = min(kTimeTile, si.T - t0);
            __syncthreads();
            for (int t = tid; t < tt; t += kThreads) time_coefficients(a, si, t0 + t, coef_s + 2 * t);
            __syncthreads();

            const int ngroups = tt * ncb;
            for (int gbase = warp * 8; gbase < ngroups; gbase += (kThreads / 32) * 8) {
                const int grp = gbase + g_in_warp;
                const bool active = grp < ngroups;
                const int gg = active ? grp : 0;
                const int t = gg / ncb, cb = gg - t * ncb;
                const int cfirst = cb * kCB;
                const float4 c0 = coef_s[2 * t], c1 = coef_s[2 * t + 1];
                float kap[kCB];
#pragma unroll
                for (int j = 0; j < kCB; ++j) kap[j] = (cfirst + j < nc) ? kappa_s[cfirst + j] : 0.f;
                cf acc[kCB][4];
#pragma unroll
                for (int j = 0; j < kCB; ++j)
#pragma unroll
                    for (int p = 0; p < 4; ++p) acc[j][p] = {0.f, 0.f};

                for (int i = part; i < np; i += kLanesPerGroup) {
                    const float4 pa = pix_s[2 * i], pb = pix_s[2 * i + 1];
                    const float4 g = geo_s[i];
                    const float tau0 = frac_turns(fmaf(c0.x, g.x, fmaf(c0.y, g.y, c0.z * g.z)));
                    const float Q = fmaf(c0.w, g.x, fmaf(c1.x, g.y, c1.y * g.z));
#pragma unroll
                    for (int j = 0; j < kCB; ++j) {
                        const float r = frac_turns(fmaf(kap[j], Q, tau0));
                        float sn, cs;
                        sincos_turns(r, &sn, &cs);
                        // pixel * exp(-i 2 pi tau)
                        cmac(acc[j][0], {pa.x, pa.y}, cs, -sn);
                        cmac(acc[j][1], {pa.z, pa.w}, cs, -sn);
                        cmac(acc[j][2], {pb.x, pb.y}, cs, -sn);
                        cmac(acc[j][3], {pb.z, pb.w}, cs, -sn);
                    }
                }
                // combine the 4 lanes of each group
#pragma unroll
                for (int j = 0; j < kCB; ++j)
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
#pragma unroll
                        for (int off = 1; off < kLanesPerGroup; off <<= 1) {
                            acc[j][p].re += __shfl_xor_sync(0xffffffffu, acc[j][p].re, off);
                            acc[j][p].im += __shfl_xor_sync(0xffffffffu, acc[j][p].im, off);
                        }
                    }
                if (active) {
                    float4 *row = a.vis + ((int64_t)si.row0 + t0 + t) * a.C * 2;
#pragma unroll
                    for (int j = 0; j < kCB; ++j) {
                        if ((j % kLanesPerGroup) != part) continue;
                        const int c = si.c0 + cfirst + j;
                        if (cfirst + j >= nc) continue;
                        float4 va = make_float4(acc[j][0].re, acc[j][0].im, acc[j][1].re, acc[j][1].im);
                        float4 vb = make_float4(acc[j][2].re, acc[j][2].im, acc[j][3].re, acc[j][3].im);
                        if (pbase > 0) {
                            const float4 oa = row[2 * c], ob = row[2 * c + 1];
                            va = make_float4(va.x + oa.x, va.y + oa.y, va.z + oa.z, va.w + oa.w);
                            vb = make_float4(vb.x + ob.x, vb.y + ob.y, vb.z + ob.z, vb.w + ob.w);
                        }
                        row[2 * c] = va;
                        row[2 * c + 1] = vb;
                    }
                }
            }
        }
    }
}

struct DegridSmem {
    float4 pix[2 * kPixBatch];
    float4 geo[kPixBatch];
    float4 coef[2 * kTimeTile];
};

__global__ void __launch_bounds__(kThreads) degridder_plain_kernel(KernelArgs a) {
    extern __shared__ float4 smem[];
    DegridSmem *sm = reinterpret_cast<DegridSmem *>(smem);
    float *kappa_s = reinterpret_cast<float *>(sm + 1);
    const int s = blockIdx.x;
    const SubgridInfo si = load_subgrid(a, s);
    if (!si.ok) {
        if (threadIdx.x == 0) flag_status(a.status, kStatusBadPlan);
        return;
    }
    degrid_subgrid(a, si, s, sm->pix, sm->geo, sm->coef, kappa_s);
}

} // namespace

cudaError_t launch_degridder(const KernelArgs &a, int variant, int max_nc, cudaStream_t stream) {
    const size_t smem = sizeof(DegridSmem) + (size_t)max_nc * 4 + 16;
    if (variant == IDG_VARIANT_PLAIN) {
        cudaError_t e =
            cudaFuncSetAttribute(degridder_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        degridder_plain_kernel<<<(unsigned)a.nr_subgrids, kThreads, smem, stream>>>(a);
        return cudaGetLastError();
    }
    return launch_degridder_fast(a, stream, batched_degridder_shape(a.S));
}

} // namespace idg
