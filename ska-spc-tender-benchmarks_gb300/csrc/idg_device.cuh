// idg_device.cuh -- device-side building blocks shared by the IDG kernels.
//
// Phase model.  For subgrid s with plan coordinates (X, Y, Z), pixel (x, y)
// and visibility (t, c) the reference evaluates (gridding_benchmark.cpp:99-124)
//   phase = u_off*l + v_off*m + w_off*n - k_c*(u_t*l + v_t*m + w_t*n)
// with l = (x + 1/2 - S/2)*image_size/S, u_off = (X + S/2 - G/2)*2*pi/image_size,
// w_off = 2*pi*w_step*(Z + 1/2) and n = (l^2+m^2)/(1+sqrt(1-l^2-m^2)).
// In FP32 the two halves are large and cancel, so the reference itself lands
// ~1e-4 (relative RMS) from FP64.  Here the phase is carried in turns and split
//   tau(x,y,t,c) = tau0(x,y,t) + kappa_c * Q(x,y,t)
//   tau0 = a_t*hx + b_t*hy + g_t*n ,   hx = x + 1/2 - S/2, hy likewise
//   Q    = qu_t*hx + qv_t*hy + qw_t*n, kappa_c = k_c - k_{c0}
// where the per-timestep coefficients a_t, b_t, g_t (everything that involves
// the subgrid offset and the first channel's wavenumber) are formed in FP64 and
// a_t, b_t are reduced modulo 2 (hx is a half-integer, so this changes tau by
// whole turns only).  What remains in FP32 is bounded by the subgrid's own
// uv extent, which keeps the result within ~1e-6 of the FP64 oracle.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/idg_gb300.h"

namespace idg {

constexpr float kTwoPiF = 6.28318530717958647692f;
constexpr double kTwoPi = 6.28318530717958647692;

// Device-side check word (see idg_device_status()), one per device.
enum : unsigned { kStatusBadPlan = 1u, kStatusBadShape = 2u, kStatusTimeout = 4u };

__device__ __forceinline__ void flag_status(unsigned *status, unsigned bits) {
    if (status) atomicOr(status, bits);
}

// x - rint(x) for |x| < 2^22, with round-to-nearest adds that the compiler
// may neither contract nor reassociate.
__device__ __forceinline__ float frac_turns(float x) {
    const float M = 12582912.0f; // 1.5 * 2^23
    const float r = __fsub_rn(__fadd_rn(x, M), M);
    return __fsub_rn(x, r);
}

// (cos 2*pi*r, sin 2*pi*r) for r in [-1/2, 1/2]: the argument stays inside
// [-pi, pi] where the SFU approximations hold ~4e-7 absolute error.
__device__ __forceinline__ void sincos_turns(float r, float *s, float *c) {
    __sincosf(kTwoPiF * r, s, c);
}

struct cf {
    float re, im;
};

__device__ __forceinline__ cf cmul(cf a, cf b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cf cconj(cf a) { return {a.re, -a.im}; }
__device__ __forceinline__ cf cadd(cf a, cf b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cf cscale(cf a, float s) { return {a.re * s, a.im * s}; }

// acc += v * p   (4 FFMA)
__device__ __forceinline__ void cmac(cf &acc, cf v, float pre, float pim) {
    acc.re = fmaf(v.re, pre, acc.re);
    acc.re = fmaf(-v.im, pim, acc.re);
    acc.im = fmaf(v.re, pim, acc.im);
    acc.im = fmaf(v.im, pre, acc.im);
}

// 2x2 complex products on {xx, xy, yx, yy} row-major.
__device__ __forceinline__ void matmul2(const cf *a, const cf *b, cf *c) {
    c[0] = cadd(cmul(a[0], b[0]), cmul(a[1], b[2]));
    c[1] = cadd(cmul(a[0], b[1]), cmul(a[1], b[3]));
    c[2] = cadd(cmul(a[2], b[0]), cmul(a[3], b[2]));
    c[3] = cadd(cmul(a[2], b[1]), cmul(a[3], b[3]));
}
__device__ __forceinline__ void hermitian2(const cf *a, cf *b) {
    b[0] = cconj(a[0]);
    b[1] = cconj(a[2]);
    b[2] = cconj(a[1]);
    b[3] = cconj(a[3]);
}
// P <- A1^H P A2 (the gridder's A-term, math.hpp:90-100)
__device__ __forceinline__ void aterm_gridder(cf *p, const cf *a1, const cf *a2) {
    cf h[4], t[4];
    hermitian2(a1, h);
    matmul2(h, p, t);
    matmul2(t, a2, p);
}
// P <- A1 P A2^H (the adjoint, common_gridding.cuh:82-94)
__device__ __forceinline__ void aterm_adjoint(cf *p, const cf *a1, const cf *a2) {
    cf h[4], t[4];
    matmul2(a1, p, t);
    hermitian2(a2, h);
    matmul2(t, h, p);
}

__device__ __forceinline__ void load_jones(const float4 *base, cf *j) {
    const float4 a = base[0], b = base[1];
    j[0] = {a.x, a.y};
    j[1] = {a.z, a.w};
    j[2] = {b.x, b.y};
    j[3] = {b.z, b.w};
}

// Everything a kernel needs about one call, by value in the launch.
struct KernelArgs {
    int G, S, C, nr_stations, nr_aterms, nr_w_planes;
    float image_size, w_step;
    unsigned flags;
    int64_t nr_subgrids, nr_rows;
    const idg_metadata *md;
    const idg_subgrid_ext *ext;
    const float *uvw;
    const float *wavenumbers;
    const float *taper;
    const float4 *aterms; // [..][S][S] of 2 x float4 (one Jones matrix)
    float4 *vis;          // [rows][C] of 2 x float4
    float2 *subgrids;     // [N][4][S][S]
    const int *work_list; // batched variant: subgrid order (may be NULL)
    int *work_counter;    // batched variant: dynamic scheduler (may be NULL)
    unsigned *status;     // device check word (may be NULL)
    int max_ctas;         // persistent kernels: at most this many CTAs (0 = fill the GPU)
    int share_den;        // persistent kernels: 1/share_den of the CTAs that fill the GPU (0, 1 = all)
};

// Plan entry after validation.
struct SubgridInfo {
    int row0, T, c0, c1, X, Y, Z;
    unsigned st1, st2;
    int aterm;
    bool ok;
};

__device__ __forceinline__ SubgridInfo load_subgrid(const KernelArgs &a, int s) {
    SubgridInfo si;
    const idg_metadata m = a.md[s];
    const int bo1 = a.md[0].baseline_offset;
    si.row0 = (m.baseline_offset - bo1) + m.time_offset;
    si.T = m.nr_timesteps;
    si.X = m.x;
    si.Y = m.y;
    si.Z = m.z;
    si.st1 = m.station1;
    si.st2 = m.station2;
    si.aterm = m.aterm_index;
    si.c0 = 0;
    si.c1 = a.C;
    if (a.ext) {
        si.c0 = a.ext[s].channel_begin;
        si.c1 = a.ext[s].channel_end;
    }
    si.ok = si.T >= 0 && si.row0 >= 0 && (int64_t)si.row0 + si.T <= a.nr_rows && si.st1 < (unsigned)a.nr_stations &&
            si.st2 < (unsigned)a.nr_stations && si.aterm >= 0 && si.aterm < a.nr_aterms && si.c0 >= 0 &&
            si.c1 <= a.C && si.c0 <= si.c1;
    return si;
}

// Per-timestep phase coefficients (see the header comment), 8 floats so that
// two 16-byte loads fetch one entry: {a, b, g, qu, qv, qw, -, -}.
__device__ __forceinline__ void time_coefficients(const KernelArgs &a, const SubgridInfo &si, int t, float4 *dst) {
    const float *p = a.uvw + 3 * ((int64_t)si.row0 + t);
    const double u = p[0], v = p[1], w = p[2];
    const double S = a.S;
    const double d2pi = (double)a.image_size / (S * kTwoPi); // metres -> turns per pixel step, per unit k
    const double k0 = a.wavenumbers[si.c0];
    double ca = ((double)si.X + S * 0.5 - a.G * 0.5) / S - k0 * u * d2pi;
    double cb = ((double)si.Y + S * 0.5 - a.G * 0.5) / S - k0 * v * d2pi;
    ca -= 2.0 * rint(ca * 0.5);
    cb -= 2.0 * rint(cb * 0.5);
    const double cg = (double)a.w_step * ((double)si.Z + 0.5) - k0 * w / kTwoPi;
    dst[0] = make_float4((float)ca, (float)cb, (float)cg, (float)(-u * d2pi));
    dst[1] = make_float4((float)(-v * d2pi), (float)(-w / kTwoPi), 0.f, 0.f);
}

// Pixel geometry {hx, hy, n} with n from the FP64 formula of math.hpp:31-37.
__device__ __forceinline__ float3 pixel_geometry(int q, int S, float image_size) {
    const int y = q / S, x = q - y * S;
    const double hx = (double)x + 0.5 - S * 0.5, hy = (double)y + 0.5 - S * 0.5;
    const double d = (double)image_size / S;
    const double l = hx * d, m = hy * d;
    const double tmp = l * l + m * m;
    const double n = tmp > 1.0 ? 1.0 : tmp / (1.0 + sqrt(1.0 - tmp));
    return make_float3((float)hx, (float)hy, (float)n);
}

} // namespace idg
