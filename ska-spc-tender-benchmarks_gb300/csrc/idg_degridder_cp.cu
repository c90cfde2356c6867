// idg_degridder_cp.cu -- batched degridder with CHANNEL-pair packing.
//
// Same result as idg_degridder.cu / idg_degridder_fast.cu.  The difference is
// what the two halves of a packed FP32x2 register hold.  The pixel-pair form
// (idg_degridder_fast.cu) packs two pixels, so every visibility accumulator is
// a pair of partial sums that is folded at the end: a lane needs 8 packed
// registers per channel.  Here a packed register holds two CHANNELS of one
// pixel's contribution, so each half of an accumulator is a distinct output:
//  * a lane keeps CB/2 x 8 packed accumulators for CB channels (half the
//    registers of the pixel-pair form), which leaves room for more warps;
//  * the pixel's staged operands are duplicated into both halves
//    ((re, re), (im, im), (-re, -re) per correlation, or a, a + b, b - a for
//    the Gauss form) and read with 16-byte loads;
//  * the phase of a channel pair is one packed FMA, x = (tau0, tau0) +
//    (kappa_c, kappa_c+1) * (Q, Q), with tau0 and Q computed once per pixel and
//    group in scalar FP32 from the FP64-derived per-timestep coefficients.
// Work split: a visibility group is one timestep x CB channels; the four lanes
// of a group each sum a quarter of the staged pixels; their partial sums are
// combined with two levels of 64-bit warp shuffles and each lane writes CB/4
// channels.
// The mirror-quad degridder (degridder_quad_kernel, below) keeps this work
// split and channel packing but stages quads of pixels (+-hx, +-hy) instead of
// pixels: its MACs share each quad's phase factors (see its section).
#include "idg_device.cuh"
#include "idg_internal.h"
#include "idg_ptx.cuh"

namespace idg {

namespace {

constexpr int kLanes = 4;             // lanes per visibility group
constexpr int kGroupsPerWarp = 32 / kLanes;
constexpr int kTimeTile = 64;
constexpr int kMaxCB = 16;
constexpr float kFastBound = 48.f;
constexpr int kGaussCp = 4;           // FLAGS bit: three-multiplication MACs

constexpr float kInv2Pi = 0.159154943091895335769f;
constexpr float k2PiHi = 6.28125f;
constexpr float k2PiLo = 1.9353071795864769253e-3f;

struct Head {
    int next, fast, qmax_bits, kmax_bits;
};

struct Layout {
    size_t pix, geo, coef, kappa, total;
};

__host__ __device__ inline Layout layout(int S, int C, int batch) {
    Layout L;
    size_t off = 64;
    L.pix = off;   off += (size_t)batch * 96;             // 12 packed operands per pixel
    L.geo = off;   off += (size_t)S * S * 16;             // (hx, hy, n, 0) per pixel
    L.coef = off;  off += (size_t)kTimeTile * 32;         // (a, b, g, qu) (qv, qw, -, -) per timestep
    L.kappa = off; off += (size_t)(C + kMaxCB) * 4;       // kappa per channel, zero padded
    L.total = (off + 15) & ~size_t(15);
    return L;
}

// x - 2 pi rint(x / 2 pi) (Cody-Waite, two constants)
__device__ __forceinline__ float reduce_2pi_s(float x) {
    const float k = rintf(x * kInv2Pi);
    return fmaf(k, -k2PiLo, fmaf(k, -k2PiHi, x));
}
__device__ __forceinline__ f2 reduce_2pi(f2 x) {
    const f2 M = pack2(12582912.0f, 12582912.0f);
    f2 k = fmul2(x, pack2(kInv2Pi, kInv2Pi));
    k = fsub2(fadd2(k, M), M);
    x = ffma2(k, pack2(-k2PiHi, -k2PiHi), x);
    return ffma2(k, pack2(-k2PiLo, -k2PiLo), x);
}

__device__ __forceinline__ f2 neg2(f2 v) { return v ^ 0x8000000080000000ull; }

__device__ __forceinline__ void sincos_pair(f2 x, f2 &c, f2 &s) {
    float x0, x1, s0, c0, s1, c1;
    unpack2(x, x0, x1);
    __sincosf(x0, &s0, &c0);
    __sincosf(x1, &s1, &c1);
    c = pack2(c0, c1);
    s = pack2(s0, s1);
}

// One pixel's contribution to the group's channel pairs.
// Four-multiplication form, V += P (cos - i sin): re += pr c + pi s, im += pi c - pr s;
// operands o[3k] = (pr, pr), o[3k+1] = (pi, pi), o[3k+2] = (-pr, -pr).
// Gauss form: k1 = pr (cos - sin), -k2 = (pr + pi) sin, k3 = (pi - pr) cos,
// Re = k1 + (-k2), Im = k1 + k3; operands a, a + b, b - a.
template <int NPAIR, bool FAST, bool GAUSS, int NACC>
__device__ __forceinline__ void pixel_macs(f2 (&acc)[NPAIR][NACC], const f2 (&kp)[NPAIR], f2 tau2, f2 Q2,
                                           uint32_t ops_addr) {
    f2 o[12];
#pragma unroll
    for (int q = 0; q < 6; ++q) lds2(ops_addr + 16 * q, o[2 * q], o[2 * q + 1]);
#pragma unroll
    for (int j = 0; j < NPAIR; ++j) {
        f2 x = ffma2(kp[j], Q2, tau2);
        if (!FAST) x = reduce_2pi(x);
        f2 C, Sn;
        sincos_pair(x, C, Sn);
        if (GAUSS) {
            const f2 cms = fsub2(C, Sn);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                acc[j][3 * k] = ffma2(o[3 * k], cms, acc[j][3 * k]);
                acc[j][3 * k + 1] = ffma2(o[3 * k + 1], Sn, acc[j][3 * k + 1]);
                acc[j][3 * k + 2] = ffma2(o[3 * k + 2], C, acc[j][3 * k + 2]);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                acc[j][2 * k] = ffma2(o[3 * k + 1], Sn, ffma2(o[3 * k], C, acc[j][2 * k]));
                acc[j][2 * k + 1] = ffma2(o[3 * k + 2], Sn, ffma2(o[3 * k + 1], C, acc[j][2 * k + 1]));
            }
        }
    }
}

template <int NPAIR, bool FAST, bool GAUSS, int NACC, int UNR>
__device__ __forceinline__ void group_pixels(f2 (&acc)[NPAIR][NACC], const f2 (&kp)[NPAIR], float A, float B, float Gc,
                                             float qu, float qv, float qw, const float4 *geo, uint32_t pix_addr,
                                             int pb, int part, int np) {
#pragma unroll UNR
    for (int i = part; i < np; i += kLanes) {
        const float4 g = geo[pb + i];
        const float tau0 = reduce_2pi_s(fmaf(A, g.x, fmaf(B, g.y, Gc * g.z)));
        const float Q = fmaf(qu, g.x, fmaf(qv, g.y, qw * g.z));
        pixel_macs<NPAIR, FAST, GAUSS, NACC>(acc, kp, pack2(tau0, tau0), pack2(Q, Q), pix_addr + 96u * (uint32_t)i);
    }
}

// Per-timestep phase coefficients of one time tile (FP64, offsets reduced,
// stored as floats: (a, b, g, qu) (qv, qw, -, -)), and the tile's decision for
// the unreduced sincos: the phase-slope bound is the sum of the three slopes
// (QSUM, one phase per pixel) or their maximum (the factored quad form).
// Contains the tile's barriers; returns the decision.
template <int NT, bool QSUM>
__device__ __forceinline__ bool tile_coefficients(const KernelArgs &a, const SubgridInfo &si, Head *head,
                                                  float4 *coef, int t0, int tt, double kref, double d2pi, float hmax,
                                                  float nmax) {
    const int tid = threadIdx.x, S = a.S;
    __syncthreads();
    for (int t = tid; t < tt; t += NT) {
        const float *p = a.uvw + 3 * ((int64_t)si.row0 + t0 + t);
        const double u = p[0], v = p[1], w = p[2];
        double ca = ((double)si.X + S * 0.5 - a.G * 0.5) / S - kref * u * d2pi;
        double cbv = ((double)si.Y + S * 0.5 - a.G * 0.5) / S - kref * v * d2pi;
        ca -= 2.0 * rint(ca * 0.5);
        cbv -= 2.0 * rint(cbv * 0.5);
        const double cg = kTwoPi * (double)a.w_step * ((double)si.Z + 0.5) - kref * w;
        const float qu = (float)(-u * d2pi * kTwoPi), qv = (float)(-v * d2pi * kTwoPi), qw = (float)(-w);
        coef[2 * t + 0] = make_float4((float)(kTwoPi * ca), (float)(kTwoPi * cbv), (float)cg, qu);
        coef[2 * t + 1] = make_float4(qv, qw, 0.f, 0.f);
        const float qm = QSUM ? fabsf(qu) * hmax + fabsf(qv) * hmax + fabsf(qw) * nmax
                              : fmaxf(fmaxf(fabsf(qu) * hmax, fabsf(qv) * hmax), fabsf(qw) * nmax);
        atomicMax(&head->qmax_bits, __float_as_int(qm));
    }
    __syncthreads();
    if (tid == 0) {
        head->fast = (3.1416f + __int_as_float(head->kmax_bits) * __int_as_float(head->qmax_bits)) <= kFastBound;
        head->qmax_bits = 0;
    }
    __syncthreads();
    return head->fast != 0;
}

// Writes a visibility group's combined sums: lane `part` stores the channel
// pairs j = part, part + 4, ... of the group (out[j][r]: correlation r / 2,
// re / im for r even / odd, the two channels in the halves), adding to the
// row when an earlier pixel batch of the subgrid already wrote it.
template <int NP>
__device__ __forceinline__ void write_group(const KernelArgs &a, const SubgridInfo &si, int t_abs, int cfirst, int nc,
                                            int part, bool accumulate, const f2 (&out)[NP][8]) {
    float4 *row = a.vis + (int64_t)t_abs * a.C * 2;
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        if (j % kLanes != part) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (cfirst + 2 * j + h >= nc) continue;
            const int c = si.c0 + cfirst + 2 * j + h;
            float w[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float lo, hi;
                unpack2(out[j][r], lo, hi);
                w[r] = h ? hi : lo;
            }
            float4 va = make_float4(w[0], w[1], w[2], w[3]);
            float4 vb = make_float4(w[4], w[5], w[6], w[7]);
            if (accumulate) {
                const float4 oa = row[2 * c], ob = row[2 * c + 1];
                va = make_float4(va.x + oa.x, va.y + oa.y, va.z + oa.z, va.w + oa.w);
                vb = make_float4(vb.x + ob.x, vb.y + ob.y, vb.z + ob.z, vb.w + ob.w);
            }
            row[2 * c] = va;
            row[2 * c + 1] = vb;
        }
    }
}

// NT threads, BATCH pixels staged per pass, at least MINB CTAs per SM, CB
// channels per group (8 or 16), FLAGS: kGaussCp; UNR: pixel-loop unrolling.
template <int NT, int BATCH, int MINB, int CB, int FLAGS, int UNR>
__global__ void __launch_bounds__(NT, MINB) degridder_cp_kernel(KernelArgs a) {
    constexpr int kT = NT, kCB = CB, kNP = CB / 2;
    constexpr bool kG = (FLAGS & kGaussCp) != 0;
    constexpr int kAcc = kG ? 12 : 8;
    static_assert(CB == 8 || CB == 16, "channel groups of 8 or 16");
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = a.S, S2 = S * S;
    const Layout L = layout(S, a.C, BATCH);
    Head *head = reinterpret_cast<Head *>(smem);
    float4 *pix = reinterpret_cast<float4 *>(smem + L.pix);
    float4 *geo = reinterpret_cast<float4 *>(smem + L.geo);
    float4 *coef = reinterpret_cast<float4 *>(smem + L.coef);
    float *kap = reinterpret_cast<float *>(smem + L.kappa);
    const uint32_t pix_addr = smem_addr(pix);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gw = lane / kLanes, part = lane % kLanes;
    const bool refcpu = (a.flags & IDG_FLAG_DEGRID_ATERM_REFCPU) != 0;
    const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;

    for (int q = tid; q < S2; q += kT) {
        const float3 g = pixel_geometry(q, S, a.image_size);
        geo[q] = make_float4(g.x, g.y, g.z, 0.f);
    }
    const double d2pi = (double)a.image_size / (double)S / kTwoPi;
    const float hmax = 0.5f * (float)(S - 1);
    const float nmax = pixel_geometry(0, S, a.image_size).z;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            head->next = atomicAdd(a.work_counter, 1);
            head->kmax_bits = 0;
            head->qmax_bits = 0;
        }
        __syncthreads();
        const int idx = head->next;
        if (idx >= a.nr_subgrids) break;
        const int s = a.work_list ? a.work_list[idx] : idx;
        const SubgridInfo si = load_subgrid(a, s);
        if (!si.ok) {
            if (tid == 0) flag_status(a.status, kStatusBadPlan);
            continue;
        }
        const int nc = si.c1 - si.c0;
        const int ncb = (nc + kCB - 1) / kCB;
        const int cref = si.c0 + (nc > 0 ? (nc - 1) / 2 : 0);
        const double kref = nc > 0 ? (double)a.wavenumbers[cref] : 0.0;
        float kmax = 0.f;
        for (int c = tid; c < ncb * kCB; c += kT) {
            float kv = 0.f;
            if (c < nc) kv = (float)((double)a.wavenumbers[si.c0 + c] - kref);
            kap[c] = kv;
            kmax = fmaxf(kmax, fabsf(kv));
        }
        if (kmax > 0.f) atomicMax(&head->kmax_bits, __float_as_int(kmax));
        const size_t jones_stride = (size_t)S2 * 2;
        const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
        const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;

        for (int pb = 0; pb < S2; pb += BATCH) {
            const int np = min(BATCH, S2 - pb);
            __syncthreads(); // previous batch consumed
            // ---- stage prepared pixels (A-terms and taper applied), operands duplicated
            for (int i = tid; i < np; i += kT) {
                const int q = pb + i;
                const float sph = taper ? a.taper[q] : 1.f;
                cf v[4];
#pragma unroll
                for (int pol = 0; pol < 4; ++pol) {
                    const float2 x = a.subgrids[((size_t)s * 4 + pol) * S2 + q];
                    v[pol] = {sph * x.x, sph * x.y};
                }
                cf j1[4], j2[4];
                load_jones(a1 + 2 * q, j1);
                load_jones(a2 + 2 * q, j2);
                if (refcpu)
                    aterm_gridder(v, j1, j2);
                else
                    aterm_adjoint(v, j1, j2);
                float e[12];
#pragma unroll
                for (int pol = 0; pol < 4; ++pol) {
                    if (kG) {
                        e[3 * pol] = v[pol].re;
                        e[3 * pol + 1] = v[pol].re + v[pol].im;
                        e[3 * pol + 2] = v[pol].im - v[pol].re;
                    } else {
                        e[3 * pol] = v[pol].re;
                        e[3 * pol + 1] = v[pol].im;
                        e[3 * pol + 2] = -v[pol].re;
                    }
                }
                float4 *d = pix + 6 * i;
#pragma unroll
                for (int r = 0; r < 6; ++r) d[r] = make_float4(e[2 * r], e[2 * r], e[2 * r + 1], e[2 * r + 1]);
            }

            for (int t0 = 0; t0 < si.T; t0 += kTimeTile) {
                const int tt = min(kTimeTile, si.T - t0);
                const bool fast = tile_coefficients<kT, true>(a, si, head, coef, t0, tt, kref, d2pi, hmax, nmax);
                const int ngroups = tt * ncb;
                for (int gbase = warp * kGroupsPerWarp; gbase < ngroups; gbase += (kT / 32) * kGroupsPerWarp) {
                    const int grp = gbase + gw;
                    const bool active = grp < ngroups;
                    const int gg = active ? grp : 0;
                    const int t = gg / ncb, cfirst = (gg - t * ncb) * kCB;
                    const float4 c0 = coef[2 * t], c1 = coef[2 * t + 1];
                    f2 kp[kNP];
#pragma unroll
                    for (int j = 0; j < kNP; ++j) kp[j] = pack2(kap[cfirst + 2 * j], kap[cfirst + 2 * j + 1]);
                    f2 acc[kNP][kAcc];
#pragma unroll
                    for (int j = 0; j < kNP; ++j)
#pragma unroll
                        for (int r = 0; r < kAcc; ++r) acc[j][r] = 0ull;
                    if (fast)
                        group_pixels<kNP, true, kG, kAcc, UNR>(acc, kp, c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, geo,
                                                               pix_addr, pb, part, np);
                    else
                        group_pixels<kNP, false, kG, kAcc, UNR>(acc, kp, c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, geo,
                                                                pix_addr, pb, part, np);
                    // combine the four lanes: both halves of a register are distinct channels
                    f2 out[kNP][8];
#pragma unroll
                    for (int j = 0; j < kNP; ++j)
#pragma unroll
                        for (int r = 0; r < 8; ++r) {
                            f2 v = kG ? fadd2(acc[j][3 * (r / 2)], acc[j][3 * (r / 2) + 1 + (r & 1)]) : acc[j][r];
                            v = fadd2(v, __shfl_xor_sync(0xffffffffu, v, 1));
                            v = fadd2(v, __shfl_xor_sync(0xffffffffu, v, 2));
                            out[j][r] = v;
                        }
                    if (active) write_group<kNP>(a, si, si.row0 + t0 + t, cfirst, nc, part, pb > 0, out);
                }
            }
        }
    }
}

template <int NT, int BATCH, int MINB, int CB, int FLAGS, int UNR>
cudaError_t launch_cp(const KernelArgs &a, cudaStream_t stream) {
    auto kern = degridder_cp_kernel<NT, BATCH, MINB, CB, FLAGS, UNR>;
    const size_t smem = layout(a.S, a.C, BATCH).total;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    if (a.share_den > 1) blocks = blocks / a.share_den > 0 ? blocks / a.share_den : 1;
    if (a.max_ctas > 0 && blocks > a.max_ctas) blocks = a.max_ctas;
    if (blocks > a.nr_subgrids) blocks = a.nr_subgrids;
    kern<<<(unsigned)blocks, NT, smem, stream>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Mirror-quad form of the degridder (shapes 13-17 of this family).  A quad is
// the four pixels (hx, hy), (-hx, -hy), (-hx, hy), (hx, -hy) of one n; with the
// gridder's factors P = e^{i a_c hx}, Q = e^{i b_c hy}, R = e^{i g_c n},
// X = P Q and Y = conj(P) Q, the four pixels' phasors are conj of X R,
// conj(X) R, Y R and conj(Y) R, so the quad contributes
//   V += conj(R) Z,  Z = P00 conj(X) + P11 X + P10 conj(Y) + P01 Y
// (P00 = pixel (hx, hy), P11 = (-hx, -hy), P10 = (-hx, hy), P01 = (hx, -hy)).
// With the quad's sums and differences staged once (per correlation
// s = P00 + P11, d = (P11.re - P00.re, P00.im - P11.im) and the same for the
// Y pair), Z costs 8 FMA per correlation and conj(R) Z 4: 3 per pixel and
// correlation against the Gauss form's 3 plus a sincos per pixel, with three
// sincos per quad (1.5 SFU operations per pixel-visibility instead of 2).
// Work split as the channel-pair kernel: a group is one timestep x CB channels,
// its four lanes split the staged quads, channels sit in the packed halves.
// ---------------------------------------------------------------------------
struct QuadLayout {
    size_t ops, geo, coef, kappa, total;
};
// 256 B of operands per quad padded to 272 B, so that the four lanes of a
// group (consecutive quads) read distinct banks: 68 words apart = 4 banks apart.
constexpr uint32_t kQuadStride = 272;

__host__ __device__ inline QuadLayout quad_layout(int S, int C, int batch) {
    QuadLayout L;
    size_t off = 64;
    L.ops = off;   off += (size_t)batch * kQuadStride;    // 32 packed operands per quad, padded
    L.geo = off;   off += (size_t)batch * 16;             // (hx, hy, n, 0) of the quad's (hx, hy) pixel
    L.coef = off;  off += (size_t)kTimeTile * 32;         // (a, b, g, qu) (qv, qw, -, -) per timestep
    L.kappa = off; off += (size_t)(C + kMaxCB) * 4;       // kappa per channel, zero padded
    L.total = (off + 15) & ~size_t(15);
    return L;
}

// Stages quad (gx, gy) of subgrid s: its pixels 0 = (gx, gy),
// 1 = (S-1-gx, S-1-gy), 2 = (S-1-gx, gy), 3 = (gx, S-1-gy) with taper and
// A-terms applied, as the operands the quad MACs read.  With e the sums and
// differences of the pixels that Z = P00 conj(X) + P11 X + P10 conj(Y) + P01 Y
// takes (Zr = Xr e0 + Xi e1 + Yr e2 + Yi e3, Zi likewise with e4..e7), and
// Xr = m1 - m2, Yr = m1 + m2, Xi = m3 + m4, Yi = m3 - m4 for the products
// m1 = Pc Qc, m2 = Ps Qs, m3 = Pc Qs, m4 = Ps Qc, the operands are
// f = (e0 + e2, e2 - e0, e1 + e3, e1 - e3, e4 + e6, e6 - e4, e5 + e7, e5 - e7):
// Zr = m1 f0 + m2 f1 + m3 f2 + m4 f3, Zi = m1 f4 + m2 f5 + m3 f6 + m4 f7.
// Correlation k's eight operands go to d[kstride * k + r], r < 4, each float4
// two operands, each duplicated into both packed halves.
__device__ __forceinline__ void stage_quad(const KernelArgs &a, int s, int gx, int gy, const float4 *a1,
                                           const float4 *a2, bool taper, bool refcpu, float4 *d, int kstride) {
    const int S = a.S, S2 = S * S;
    const int qx[4] = {gx, S - 1 - gx, S - 1 - gx, gx};
    const int qy[4] = {gy, S - 1 - gy, gy, S - 1 - gy};
    cf v[4][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int q = qy[e] * S + qx[e];
        const float sph = taper ? a.taper[q] : 1.f;
#pragma unroll
        for (int pol = 0; pol < 4; ++pol) {
            const float2 x = a.subgrids[((size_t)s * 4 + pol) * S2 + q];
            v[e][pol] = {sph * x.x, sph * x.y};
        }
        cf j1[4], j2[4];
        load_jones(a1 + 2 * q, j1);
        load_jones(a2 + 2 * q, j2);
        if (refcpu)
            aterm_gridder(v[e], j1, j2);
        else
            aterm_adjoint(v[e], j1, j2);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const cf p00 = v[0][k], p11 = v[1][k], p10 = v[2][k], p01 = v[3][k];
        const float e[8] = {p00.re + p11.re, p00.im - p11.im, p10.re + p01.re, p10.im - p01.im,
                            p00.im + p11.im, p11.re - p00.re, p10.im + p01.im, p01.re - p10.re};
        const float f[8] = {e[0] + e[2], e[2] - e[0], e[1] + e[3], e[1] - e[3],
                            e[4] + e[6], e[6] - e[4], e[5] + e[7], e[5] - e[7]};
#pragma unroll
        for (int r = 0; r < 4; ++r)
            d[kstride * k + r] = make_float4(f[2 * r], f[2 * r], f[2 * r + 1], f[2 * r + 1]);
    }
}

// KP: the channel pairs' kappa, either f2 registers (f2[NPAIR]) or a pointer
// to the group's first channel in shared memory (read per channel pair).
__device__ __forceinline__ f2 kappa_pair(const f2 (&kp)[4], int j) { return kp[j]; }
__device__ __forceinline__ f2 kappa_pair(const float *kp, int j) {
    return *reinterpret_cast<const f2 *>(kp + 2 * j);
}

template <int NPAIR, bool FAST, typename KP>
__device__ __forceinline__ void quad_macs(f2 (&acc)[NPAIR][4][2], const KP &kp, float4 g, float A, float B,
                                          float Gc, float qu, float qv, float qw, uint32_t ops_addr) {
    const float tx = reduce_2pi_s(A * g.x), ty = reduce_2pi_s(B * g.y), tn = reduce_2pi_s(Gc * g.z);
    const f2 TX = pack2(tx, tx), TY = pack2(ty, ty), TN = pack2(tn, tn);
    const float qx = qu * g.x, qy = qv * g.y, qn = qw * g.z;
    const f2 QX = pack2(qx, qx), QY = pack2(qy, qy), QN = pack2(qn, qn);
    // per correlation k: o[8k..8k+7] = (s_r, d_i, s'_r, d'_i, s_i, d_r, s'_i, d'_r), each duplicated
    f2 o[32];
#pragma unroll
    for (int q = 0; q < 16; ++q) lds2(ops_addr + 16 * q, o[2 * q], o[2 * q + 1]);
#pragma unroll
    for (int j = 0; j < NPAIR; ++j) {
        const f2 kj = kappa_pair(kp, j);
        f2 ap = ffma2(kj, QX, TX), aq = ffma2(kj, QY, TY), ar = ffma2(kj, QN, TN);
        if (!FAST) {
            ap = reduce_2pi(ap);
            aq = reduce_2pi(aq);
            ar = reduce_2pi(ar);
        }
        f2 Pc, Ps, Qc, Qs, Rc, Rs;
        sincos_pair(ap, Pc, Ps);
        sincos_pair(aq, Qc, Qs);
        sincos_pair(ar, Rc, Rs);
        const f2 nRs = neg2(Rs);
        const f2 m1 = fmul2(Pc, Qc), m2 = fmul2(Ps, Qs), m3 = fmul2(Pc, Qs), m4 = fmul2(Ps, Qc);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const f2 *p = o + 8 * k;
            const f2 Zr = ffma2(m4, p[3], ffma2(m3, p[2], ffma2(m2, p[1], fmul2(m1, p[0]))));
            const f2 Zi = ffma2(m4, p[7], ffma2(m3, p[6], ffma2(m2, p[5], fmul2(m1, p[4]))));
            // V += conj(R) Z
            acc[j][k][0] = ffma2(Rs, Zi, ffma2(Rc, Zr, acc[j][k][0]));
            acc[j][k][1] = ffma2(nRs, Zr, ffma2(Rc, Zi, acc[j][k][1]));
        }
    }
}

// Column form (COL): quads are staged column by column (slot i of a batch is
// quad qb + i in column-major order), so the slots a lane visits (i, i + 4, ...)
// run down one column for Sh / 4 steps when Sh is a multiple of 4.  P depends
// on hx only: a lane computes it when its quad's hx changes and keeps it
// (Pc, Ps per channel pair, 16 registers) for the next quads, which leaves two
// sincos per quad and channel (Q and R) plus P once per column run.  The MACs
// are those of quad_macs.  The extra registers need the uncapped budget of
// 8 warps per SM; at 12 warps the spills cost more than the saved sincos.
template <int NPAIR, bool FAST, typename KP>
__device__ __forceinline__ void column_factors(f2 (&Pc)[NPAIR], f2 (&Ps)[NPAIR], const KP &kp, float hx, float A,
                                               float qu) {
    const float tx = reduce_2pi_s(A * hx), qx = qu * hx;
    const f2 TX = pack2(tx, tx), QX = pack2(qx, qx);
#pragma unroll
    for (int j = 0; j < NPAIR; ++j) {
        f2 ap = ffma2(kappa_pair(kp, j), QX, TX);
        if (!FAST) ap = reduce_2pi(ap);
        sincos_pair(ap, Pc[j], Ps[j]);
    }
}

template <int NPAIR, bool FAST, typename KP>
__device__ __forceinline__ void quad_macs_col(f2 (&acc)[NPAIR][4][2], const f2 (&Pc)[NPAIR], const f2 (&Ps)[NPAIR],
                                              const KP &kp, float4 g, float B, float Gc, float qv, float qw,
                                              uint32_t ops_addr) {
    const float ty = reduce_2pi_s(B * g.y), tn = reduce_2pi_s(Gc * g.z);
    const f2 TY = pack2(ty, ty), TN = pack2(tn, tn);
    const float qy = qv * g.y, qn = qw * g.z;
    const f2 QY = pack2(qy, qy), QN = pack2(qn, qn);
    f2 o[32];
#pragma unroll
    for (int q = 0; q < 16; ++q) lds2(ops_addr + 16 * q, o[2 * q], o[2 * q + 1]);
#pragma unroll
    for (int j = 0; j < NPAIR; ++j) {
        const f2 kj = kappa_pair(kp, j);
        f2 aq = ffma2(kj, QY, TY), ar = ffma2(kj, QN, TN);
        if (!FAST) {
            aq = reduce_2pi(aq);
            ar = reduce_2pi(ar);
        }
        f2 Qc, Qs, Rc, Rs;
        sincos_pair(aq, Qc, Qs);
        sincos_pair(ar, Rc, Rs);
        const f2 nRs = neg2(Rs);
        const f2 m1 = fmul2(Pc[j], Qc), m2 = fmul2(Ps[j], Qs), m3 = fmul2(Pc[j], Qs), m4 = fmul2(Ps[j], Qc);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const f2 *p = o + 8 * k;
            const f2 Zr = ffma2(m4, p[3], ffma2(m3, p[2], ffma2(m2, p[1], fmul2(m1, p[0]))));
            const f2 Zi = ffma2(m4, p[7], ffma2(m3, p[6], ffma2(m2, p[5], fmul2(m1, p[4]))));
            acc[j][k][0] = ffma2(Rs, Zi, ffma2(Rc, Zr, acc[j][k][0]));
            acc[j][k][1] = ffma2(nRs, Zr, ffma2(Rc, Zi, acc[j][k][1]));
        }
    }
}

// Phasors first (PF): the quad's factors X, Y, R of every channel pair are
// formed before any MAC -- all the pairs' sincos are independent and in
// flight together -- and the operands are then read one correlation at a
// time, each used by every channel pair.  Same arithmetic as quad_macs_col.
template <int NPAIR, bool FAST, typename KP>
__device__ __forceinline__ void quad_macs_col_pf(f2 (&acc)[NPAIR][4][2], const f2 (&Pc)[NPAIR],
                                                 const f2 (&Ps)[NPAIR], const KP &kp, float4 g, float B, float Gc,
                                                 float qv, float qw, uint32_t ops_addr) {
    const float ty = reduce_2pi_s(B * g.y), tn = reduce_2pi_s(Gc * g.z);
    const f2 TY = pack2(ty, ty), TN = pack2(tn, tn);
    const float qy = qv * g.y, qn = qw * g.z;
    const f2 QY = pack2(qy, qy), QN = pack2(qn, qn);
    f2 m1[NPAIR], m2[NPAIR], m3[NPAIR], m4[NPAIR], Rc[NPAIR], Rs[NPAIR];
#pragma unroll
    for (int j = 0; j < NPAIR; ++j) {
        const f2 kj = kappa_pair(kp, j);
        f2 aq = ffma2(kj, QY, TY), ar = ffma2(kj, QN, TN);
        if (!FAST) {
            aq = reduce_2pi(aq);
            ar = reduce_2pi(ar);
        }
        f2 Qc, Qs;
        sincos_pair(aq, Qc, Qs);
        sincos_pair(ar, Rc[j], Rs[j]);
        m1[j] = fmul2(Pc[j], Qc);
        m2[j] = fmul2(Ps[j], Qs);
        m3[j] = fmul2(Pc[j], Qs);
        m4[j] = fmul2(Ps[j], Qc);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        f2 p[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) lds2(ops_addr + 64 * k + 16 * q, p[2 * q], p[2 * q + 1]);
#pragma unroll
        for (int j = 0; j < NPAIR; ++j) {
            const f2 Zr = ffma2(m4[j], p[3], ffma2(m3[j], p[2], ffma2(m2[j], p[1], fmul2(m1[j], p[0]))));
            const f2 Zi = ffma2(m4[j], p[7], ffma2(m3[j], p[6], ffma2(m2[j], p[5], fmul2(m1[j], p[4]))));
            acc[j][k][0] = ffma2(Rs[j], Zi, ffma2(Rc[j], Zr, acc[j][k][0]));
            acc[j][k][1] = ffma2(neg2(Rs[j]), Zr, ffma2(Rc[j], Zi, acc[j][k][1]));
        }
    }
}

template <int NPAIR, bool FAST, bool PF, typename KP>
__device__ __forceinline__ void quad_col(f2 (&acc)[NPAIR][4][2], const f2 (&Pc)[NPAIR], const f2 (&Ps)[NPAIR],
                                         const KP &kp, float4 g, float4 c0, float4 c1, uint32_t addr) {
    if (PF)
        quad_macs_col_pf<NPAIR, FAST>(acc, Pc, Ps, kp, g, c0.y, c0.z, c1.x, c1.y, addr);
    else
        quad_macs_col<NPAIR, FAST>(acc, Pc, Ps, kp, g, c0.y, c0.z, c1.x, c1.y, addr);
}

template <int NPAIR, bool FAST, bool PF, typename KP>
__device__ __forceinline__ void column_loop(f2 (&acc)[NPAIR][4][2], const KP &kp, const float4 *geo, float4 c0,
                                            float4 c1, uint32_t ops_addr, int part, int nq) {
    f2 Pc[NPAIR], Ps[NPAIR];
    float cur = __int_as_float(0x7fc00000); // NaN: the first quad always computes P
    for (int i = part; i < nq; i += kLanes) {
        const float4 g = geo[i];
        if (!(g.x == cur)) {
            cur = g.x;
            column_factors<NPAIR, FAST>(Pc, Ps, kp, g.x, c0.x, c0.w);
        }
        quad_col<NPAIR, FAST, PF>(acc, Pc, Ps, kp, g, c0, c1, ops_addr + kQuadStride * (uint32_t)i);
    }
}

// Column runs of known length (RUN > 0): when every column of the batch holds
// kLanes * RUN quads and the batch starts on a column, a lane's quads come in
// runs of RUN down one column; P is formed once per run and the run's quads
// are one straight-line block (no per-quad test of hx).
template <int NPAIR, bool FAST, bool PF, int RUN, typename KP>
__device__ __forceinline__ void column_loop_runs(f2 (&acc)[NPAIR][4][2], const KP &kp, const float4 *geo, float4 c0,
                                                 float4 c1, uint32_t ops_addr, int part, int nq) {
    f2 Pc[NPAIR], Ps[NPAIR];
    for (int i0 = part; i0 < nq; i0 += kLanes * RUN) {
        column_factors<NPAIR, FAST>(Pc, Ps, kp, geo[i0].x, c0.x, c0.w);
#pragma unroll
        for (int u = 0; u < RUN; ++u) {
            const int i = i0 + kLanes * u;
            quad_col<NPAIR, FAST, PF>(acc, Pc, Ps, kp, geo[i], c0, c1, ops_addr + kQuadStride * (uint32_t)i);
        }
    }
}

// COL: the column form (column_loop); otherwise quads row by row.
// RUN > 0: the column form's runs of RUN quads as straight-line blocks, where
// the batch's columns hold exactly kLanes * RUN quads.  PF: phasors first.
template <int NT, int QB, int CB, int UNR, bool KSM, bool COL, int RUN, bool PF>
__device__ __forceinline__ void degridder_quad_body(const KernelArgs &a) {
    constexpr int kT = NT, kCB = CB, kNP = CB / 2;
    static_assert(CB == 4 || CB == 8, "channel groups of 4 or 8");
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = a.S, S2 = S * S, Sh = S / 2, nquads = Sh * Sh;
    const QuadLayout L = quad_layout(S, a.C, QB);
    Head *head = reinterpret_cast<Head *>(smem);
    float4 *ops = reinterpret_cast<float4 *>(smem + L.ops);
    float4 *geo = reinterpret_cast<float4 *>(smem + L.geo);
    float4 *coef = reinterpret_cast<float4 *>(smem + L.coef);
    float *kap = reinterpret_cast<float *>(smem + L.kappa);
    const uint32_t ops_addr = smem_addr(ops);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gw = lane / kLanes, part = lane % kLanes;
    const bool refcpu = (a.flags & IDG_FLAG_DEGRID_ATERM_REFCPU) != 0;
    const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;
    const double d2pi = (double)a.image_size / (double)S / kTwoPi;
    const float hmax = 0.5f * (float)(S - 1);
    const float nmax = pixel_geometry(0, S, a.image_size).z;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            head->next = atomicAdd(a.work_counter, 1);
            head->kmax_bits = 0;
            head->qmax_bits = 0;
        }
        __syncthreads();
        const int idx = head->next;
        if (idx >= a.nr_subgrids) break;
        const int s = a.work_list ? a.work_list[idx] : idx;
        const SubgridInfo si = load_subgrid(a, s);
        if (!si.ok) {
            if (tid == 0) flag_status(a.status, kStatusBadPlan);
            continue;
        }
        const int nc = si.c1 - si.c0;
        const int ncb = (nc + kCB - 1) / kCB;
        const int cref = si.c0 + (nc > 0 ? (nc - 1) / 2 : 0);
        const double kref = nc > 0 ? (double)a.wavenumbers[cref] : 0.0;
        float kmax = 0.f;
        for (int c = tid; c < ncb * kCB; c += kT) {
            float kv = 0.f;
            if (c < nc) kv = (float)((double)a.wavenumbers[si.c0 + c] - kref);
            kap[c] = kv;
            kmax = fmaxf(kmax, fabsf(kv));
        }
        if (kmax > 0.f) atomicMax(&head->kmax_bits, __float_as_int(kmax));
        const size_t jones_stride = (size_t)S2 * 2;
        const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
        const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;

        for (int qb = 0; qb < nquads; qb += QB) {
            const int nq = min(QB, nquads - qb);
            __syncthreads(); // previous batch consumed
            // ---- stage the batch's quads: A-terms and taper applied, sums and differences
            for (int i = tid; i < nq; i += kT) {
                const int g = qb + i;
                const int gy = COL ? g % Sh : g / Sh, gx = COL ? g / Sh : g % Sh;
                stage_quad(a, s, gx, gy, a1, a2, taper, refcpu, ops + (kQuadStride / 16) * i, 4);
                const float3 gg = pixel_geometry(gy * S + gx, S, a.image_size);
                geo[i] = make_float4(gg.x, gg.y, gg.z, 0.f);
            }

            for (int t0 = 0; t0 < si.T; t0 += kTimeTile) {
                const int tt = min(kTimeTile, si.T - t0);
                const bool fast = tile_coefficients<kT, false>(a, si, head, coef, t0, tt, kref, d2pi, hmax, nmax);
                const int ngroups = tt * ncb;
                for (int gbase = warp * kGroupsPerWarp; gbase < ngroups; gbase += (kT / 32) * kGroupsPerWarp) {
                    const int grp = gbase + gw;
                    const bool active = grp < ngroups;
                    const int gg = active ? grp : 0;
                    const int t = gg / ncb, cfirst = (gg - t * ncb) * kCB;
                    const float4 c0 = coef[2 * t], c1 = coef[2 * t + 1];
                    f2 kp[kNP];
#pragma unroll
                    for (int j = 0; j < kNP; ++j) kp[j] = pack2(kap[cfirst + 2 * j], kap[cfirst + 2 * j + 1]);
                    f2 acc[kNP][4][2];
#pragma unroll
                    for (int j = 0; j < kNP; ++j)
#pragma unroll
                        for (int k = 0; k < 4; ++k) acc[j][k][0] = acc[j][k][1] = 0ull;
                    const float *kps = kap + cfirst;
                    const bool runs = RUN > 0 && Sh == kLanes * RUN && qb % Sh == 0 && nq % Sh == 0;
                    if (COL && runs) {
                        if (fast)
                            column_loop_runs<kNP, true, PF, (RUN > 0 ? RUN : 1)>(acc, kps, geo, c0, c1, ops_addr,
                                                                                 part, nq);
                        else
                            column_loop_runs<kNP, false, PF, (RUN > 0 ? RUN : 1)>(acc, kps, geo, c0, c1, ops_addr,
                                                                                  part, nq);
                    } else if (COL) {
                        if (fast)
                            column_loop<kNP, true, PF>(acc, kps, geo, c0, c1, ops_addr, part, nq);
                        else
                            column_loop<kNP, false, PF>(acc, kps, geo, c0, c1, ops_addr, part, nq);
                    } else if (fast) {
#pragma unroll UNR
                        for (int i = part; i < nq; i += kLanes) {
                            if (KSM)
                                quad_macs<kNP, true>(acc, kps, geo[i], c0.x, c0.y, c0.z, c0.w, c1.x, c1.y,
                                                     ops_addr + kQuadStride * (uint32_t)i);
                            else
                                quad_macs<kNP, true>(acc, kp, geo[i], c0.x, c0.y, c0.z, c0.w, c1.x, c1.y,
                                                     ops_addr + kQuadStride * (uint32_t)i);
                        }
                    } else {
#pragma unroll UNR
                        for (int i = part; i < nq; i += kLanes) {
                            if (KSM)
                                quad_macs<kNP, false>(acc, kps, geo[i], c0.x, c0.y, c0.z, c0.w, c1.x, c1.y,
                                                      ops_addr + kQuadStride * (uint32_t)i);
                            else
                                quad_macs<kNP, false>(acc, kp, geo[i], c0.x, c0.y, c0.z, c0.w, c1.x, c1.y,
                                                      ops_addr + kQuadStride * (uint32_t)i);
                        }
                    }
                    // combine the four lanes
                    f2 out[kNP][8];
#pragma unroll
                    for (int j = 0; j < kNP; ++j)
#pragma unroll
                        for (int k = 0; k < 4; ++k)
#pragma unroll
                            for (int r = 0; r < 2; ++r) {
                                f2 v = acc[j][k][r];
                                v = fadd2(v, __shfl_xor_sync(0xffffffffu, v, 1));
                                v = fadd2(v, __shfl_xor_sync(0xffffffffu, v, 2));
                                out[j][2 * k + r] = v;
                            }
                    if (active) write_group<kNP>(a, si, si.row0 + t0 + t, cfirst, nc, part, qb > 0, out);
                }
            }
        }
    }
}

// The kernel: register budget from the CTAs per SM (MINB), or, with MAXR > 0,
// a fixed cap of MAXR registers per thread (for CTA sizes whose budget the
// compiler rounds down: 96-thread CTAs x 3 per SM may use 224 registers).
template <int NT, int QB, int MINB, int CB, int UNR, bool KSM, bool COL, int RUN, bool PF>
__global__ void __launch_bounds__(NT, MINB) degridder_quad_kernel(KernelArgs a) {
    degridder_quad_body<NT, QB, CB, UNR, KSM, COL, RUN, PF>(a);
}
template <int MAXR, int NT, int QB, int CB, int UNR, bool KSM, bool COL, int RUN, bool PF>
__global__ void __maxnreg__(MAXR) degridder_quad_kernel_r(KernelArgs a) {
    degridder_quad_body<NT, QB, CB, UNR, KSM, COL, RUN, PF>(a);
}

// ---------------------------------------------------------------------------
// Swap-symmetric octets (degridder_oct_kernel).  Quad (a, b) and its transpose
// (b, a) hold pixels with the same n (l and m swap), so one R = e^{i g n}
// serves eight pixels.  With quad 1 = (a, b) and quad 2 = (b, a), a < b,
//   V += conj(R) (Z1 + Z2),
// Z1 from P = P(ha), Q = Q(hb) and quad 1's operands, Z2 likewise from
// P(hb), Q(ha) and quad 2's: 8 FMA per correlation for each Z, and the
// rotation by conj(R) (4 FMA) is shared.  A correlation costs 20 FMA per
// eight pixels instead of 24; per pixel and channel 11.6 FMA (13.5 for
// quads) and 1.25 sincos (1.125).  The diagonal quads (a, a) are their own
// transposes and stay quads.
// The factors of all channel pairs are formed first (88 registers), then the
// operands are read one correlation at a time (32 registers): a whole octet's
// operands (128 registers) would not fit beside the accumulators.  Forming
// the factors two channel pairs at a time (operands read twice) needs as many
// registers, and at 12 warps per SM both forms spill heavily.
// On GB300 at S = 32 the octets run within 1 % of the column-form quads: the
// five sincos per octet and channel pair keep the SFU pipe about half busy,
// where a column run of quads needs 2.25 per quad.  The autotuner picks
// between them per subgrid size.
// ---------------------------------------------------------------------------
// 512 B of operands per octet padded to 528 B: the four lanes of a group read
// octets 132 words = 4 banks apart.
constexpr uint32_t kOctStride = 528;

struct OctLayout {
    size_t ops, diag, geo, dgeo, coef, kappa, total;
    int ob;  // octets per batch
};

__host__ __device__ inline OctLayout oct_layout(int S, int C, int ob_max) {
    const int Sh = S / 2, no = Sh * (Sh - 1) / 2;
    OctLayout L;
    L.ob = no < ob_max ? no : ob_max;
    size_t off = 64;
    L.ops = off;   off += (size_t)L.ob * kOctStride;      // octet operands, per correlation quad 1 then quad 2
    L.diag = off;  off += (size_t)Sh * kQuadStride;       // the Sh diagonal quads (last batch)
    L.geo = off;   off += (size_t)L.ob * 16;              // (ha, hb, n, 0) of pixel (a, b)
    L.dgeo = off;  off += (size_t)Sh * 16;
    L.coef = off;  off += (size_t)kTimeTile * 32;         // (a, b, g, qu) (qv, qw, -, -) per timestep
    L.kappa = off; off += (size_t)(C + kMaxCB) * 4;       // kappa per channel, zero padded
    L.total = (off + 15) & ~size_t(15);
    return L;
}

// Octet index u (row-major over a < b) -> (a, b).
__device__ __forceinline__ void octet_coords(int u, int Sh, int &a, int &b) {
    int r = 0;
    while (u >= Sh - 1 - r) {
        u -= Sh - 1 - r;
        ++r;
    }
    a = r;
    b = r + 1 + u;
}

// g = (ha, hb, n, 0); c0 = (A, B, G, qu), c1 = (qv, qw, -, -).
template <int NPAIR, bool FAST>
__device__ __forceinline__ void oct_macs(f2 (&acc)[NPAIR][4][2], const float *kp, float4 g, float4 c0, float4 c1,
                                         uint32_t ops_addr) {
    const float A = c0.x, B = c0.y, Gc = c0.z, qu = c0.w, qv = c1.x, qw = c1.y;
    const float tp1 = reduce_2pi_s(A * g.x), tq1 = reduce_2pi_s(B * g.y);
    const float tp2 = reduce_2pi_s(A * g.y), tq2 = reduce_2pi_s(B * g.x);
    const float tn = reduce_2pi_s(Gc * g.z);
    const float sp1 = qu * g.x, sq1 = qv * g.y, sp2 = qu * g.y, sq2 = qv * g.x, sn = qw * g.z;
    const f2 TP1 = pack2(tp1, tp1), TQ1 = pack2(tq1, tq1), TP2 = pack2(tp2, tp2), TQ2 = pack2(tq2, tq2),
             TN = pack2(tn, tn);
    const f2 SP1 = pack2(sp1, sp1), SQ1 = pack2(sq1, sq1), SP2 = pack2(sp2, sp2), SQ2 = pack2(sq2, sq2),
             SN = pack2(sn, sn);
    f2 a1[NPAIR], a2[NPAIR], a3[NPAIR], a4[NPAIR];  // quad 1's m1..m4
    f2 b1[NPAIR], b2[NPAIR], b3[NPAIR], b4[NPAIR];  // quad 2's
    f2 Rc[NPAIR], Rs[NPAIR], nRs[NPAIR];
#pragma unroll
    for (int j = 0; j < NPAIR; ++j) {
        const f2 kj = kappa_pair(kp, j);
        f2 ap1 = ffma2(kj, SP1, TP1), aq1 = ffma2(kj, SQ1, TQ1);
        f2 ap2 = ffma2(kj, SP2, TP2), aq2 = ffma2(kj, SQ2, TQ2), ar = ffma2(kj, SN, TN);
        if (!FAST) {
            ap1 = reduce_2pi(ap1);
            aq1 = reduce_2pi(aq1);
            ap2 = reduce_2pi(ap2);
            aq2 = reduce_2pi(aq2);
            ar = reduce_2pi(ar);
        }
        f2 Pc, Ps, Qc, Qs;
        sincos_pair(ap1, Pc, Ps);
        sincos_pair(aq1, Qc, Qs);
        a1[j] = fmul2(Pc, Qc);
        a2[j] = fmul2(Ps, Qs);
        a3[j] = fmul2(Pc, Qs);
        a4[j] = fmul2(Ps, Qc);
        sincos_pair(ap2, Pc, Ps);
        sincos_pair(aq2, Qc, Qs);
        b1[j] = fmul2(Pc, Qc);
        b2[j] = fmul2(Ps, Qs);
        b3[j] = fmul2(Pc, Qs);
        b4[j] = fmul2(Ps, Qc);
        sincos_pair(ar, Rc[j], Rs[j]);
        nRs[j] = neg2(Rs[j]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        f2 p[16];
#pragma unroll
        for (int q = 0; q < 8; ++q) lds2(ops_addr + 128 * k + 16 * q, p[2 * q], p[2 * q + 1]);
#pragma unroll
        for (int j = 0; j < NPAIR; ++j) {
            f2 Zr = fmul2(a1[j], p[0]);
            Zr = ffma2(a2[j], p[1], Zr);
            Zr = ffma2(a3[j], p[2], Zr);
            Zr = ffma2(a4[j], p[3], Zr);
            Zr = ffma2(b1[j], p[8], Zr);
            Zr = ffma2(b2[j], p[9], Zr);
            Zr = ffma2(b3[j], p[10], Zr);
            Zr = ffma2(b4[j], p[11], Zr);
            f2 Zi = fmul2(a1[j], p[4]);
            Zi = ffma2(a2[j], p[5], Zi);
            Zi = ffma2(a3[j], p[6], Zi);
            Zi = ffma2(a4[j], p[7], Zi);
            Zi = ffma2(b1[j], p[12], Zi);
            Zi = ffma2(b2[j], p[13], Zi);
            Zi = ffma2(b3[j], p[14], Zi);
            Zi = ffma2(b4[j], p[15], Zi);
            acc[j][k][0] = ffma2(Rs[j], Zi, ffma2(Rc[j], Zr, acc[j][k][0]));
            acc[j][k][1] = ffma2(nRs[j], Zr, ffma2(Rc[j], Zi, acc[j][k][1]));
        }
    }
}

// Work split as in the quad kernel (a group is one timestep x CB channels,
// four lanes split the staged units).  A subgrid's Sh (Sh - 1) / 2 octets are
// staged in batches of at most OB; the last batch also holds the Sh diagonal
// quads.  S = 32: one batch of 120 octets and 16 quads, 30 + 4 per lane.
template <int NT, int OB, int CB>
__device__ __forceinline__ void degridder_oct_body(const KernelArgs &a) {
    constexpr int kT = NT, kCB = CB, kNP = CB / 2;
    static_assert(CB == 4 || CB == 8, "channel groups of 4 or 8");
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = a.S, S2 = S * S, Sh = S / 2, no = Sh * (Sh - 1) / 2;
    const OctLayout L = oct_layout(S, a.C, OB);
    const int nbatch = no > 0 ? (no + L.ob - 1) / L.ob : 1;
    Head *head = reinterpret_cast<Head *>(smem);
    float4 *ops = reinterpret_cast<float4 *>(smem + L.ops);
    float4 *dops = reinterpret_cast<float4 *>(smem + L.diag);
    float4 *geo = reinterpret_cast<float4 *>(smem + L.geo);
    float4 *dgeo = reinterpret_cast<float4 *>(smem + L.dgeo);
    float4 *coef = reinterpret_cast<float4 *>(smem + L.coef);
    float *kap = reinterpret_cast<float *>(smem + L.kappa);
    const uint32_t ops_addr = smem_addr(ops), dops_addr = smem_addr(dops);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gw = lane / kLanes, part = lane % kLanes;
    const bool refcpu = (a.flags & IDG_FLAG_DEGRID_ATERM_REFCPU) != 0;
    const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;
    const double d2pi = (double)a.image_size / (double)S / kTwoPi;
    const float hmax = 0.5f * (float)(S - 1);
    const float nmax = pixel_geometry(0, S, a.image_size).z;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            head->next = atomicAdd(a.work_counter, 1);
            head->kmax_bits = 0;
            head->qmax_bits = 0;
        }
        __syncthreads();
        const int idx = head->next;
        if (idx >= a.nr_subgrids) break;
        const int s = a.work_list ? a.work_list[idx] : idx;
        const SubgridInfo si = load_subgrid(a, s);
        if (!si.ok) {
            if (tid == 0) flag_status(a.status, kStatusBadPlan);
            continue;
        }
        const int nc = si.c1 - si.c0;
        const int ncb = (nc + kCB - 1) / kCB;
        const int cref = si.c0 + (nc > 0 ? (nc - 1) / 2 : 0);
        const double kref = nc > 0 ? (double)a.wavenumbers[cref] : 0.0;
        float kmax = 0.f;
        for (int c = tid; c < ncb * kCB; c += kT) {
            float kv = 0.f;
            if (c < nc) kv = (float)((double)a.wavenumbers[si.c0 + c] - kref);
            kap[c] = kv;
            kmax = fmaxf(kmax, fabsf(kv));
        }
        if (kmax > 0.f) atomicMax(&head->kmax_bits, __float_as_int(kmax));
        const size_t jones_stride = (size_t)S2 * 2;
        const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
        const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;

        for (int b = 0; b < nbatch; ++b) {
            const int o0 = b * L.ob;
            const int nob = no - o0 < L.ob ? no - o0 : L.ob;
            const int nd = b == nbatch - 1 ? Sh : 0;
            __syncthreads(); // previous batch consumed
            for (int i = tid; i < nob + nd; i += kT) {
                if (i < nob) {
                    int oa, ob;
                    octet_coords(o0 + i, Sh, oa, ob);
                    float4 *d = ops + (kOctStride / 16) * i;
                    stage_quad(a, s, oa, ob, a1, a2, taper, refcpu, d, 8);
                    stage_quad(a, s, ob, oa, a1, a2, taper, refcpu, d + 4, 8);
                    const float3 gg = pixel_geometry(ob * S + oa, S, a.image_size);
                    geo[i] = make_float4(gg.x, gg.y, gg.z, 0.f);
                } else {
                    const int dq = i - nob;
                    stage_quad(a, s, dq, dq, a1, a2, taper, refcpu, dops + (kQuadStride / 16) * dq, 4);
                    const float3 gg = pixel_geometry(dq * S + dq, S, a.image_size);
                    dgeo[dq] = make_float4(gg.x, gg.y, gg.z, 0.f);
                }
            }

            for (int t0 = 0; t0 < si.T; t0 += kTimeTile) {
                const int tt = min(kTimeTile, si.T - t0);
                const bool fast = tile_coefficients<kT, false>(a, si, head, coef, t0, tt, kref, d2pi, hmax, nmax);
                const int ngroups = tt * ncb;
                for (int gbase = warp * kGroupsPerWarp; gbase < ngroups; gbase += (kT / 32) * kGroupsPerWarp) {
                    const int grp = gbase + gw;
                    const bool active = grp < ngroups;
                    const int gg = active ? grp : 0;
                    const int t = gg / ncb, cfirst = (gg - t * ncb) * kCB;
                    const float4 c0 = coef[2 * t], c1 = coef[2 * t + 1];
                    f2 acc[kNP][4][2];
#pragma unroll
                    for (int j = 0; j < kNP; ++j)
#pragma unroll
                        for (int k = 0; k < 4; ++k) acc[j][k][0] = acc[j][k][1] = 0ull;
                    const float *kps = kap + cfirst;
                    if (fast) {
                        for (int i = part; i < nob; i += kLanes)
                            oct_macs<kNP, true>(acc, kps, geo[i], c0, c1, ops_addr + kOctStride * (uint32_t)i);
                        for (int i = part; i < nd; i += kLanes)
                            quad_macs<kNP, true>(acc, kps, dgeo[i], c0.x, c0.y, c0.z, c0.w, c1.x, c1.y,
                                                 dops_addr + kQuadStride * (uint32_t)i);
                    } else {
                        for (int i = part; i < nob; i += kLanes)
                            oct_macs<kNP, false>(acc, kps, geo[i], c0, c1, ops_addr + kOctStride * (uint32_t)i);
                        for (int i = part; i < nd; i += kLanes)
                            quad_macs<kNP, false>(acc, kps, dgeo[i], c0.x, c0.y, c0.z, c0.w, c1.x, c1.y,
                                                  dops_addr + kQuadStride * (uint32_t)i);
                    }
                    f2 out[kNP][8];
#pragma unroll
                    for (int j = 0; j < kNP; ++j)
#pragma unroll
                        for (int k = 0; k < 4; ++k)
#pragma unroll
                            for (int r = 0; r < 2; ++r) {
                                f2 v = acc[j][k][r];
                                v = fadd2(v, __shfl_xor_sync(0xffffffffu, v, 1));
                                v = fadd2(v, __shfl_xor_sync(0xffffffffu, v, 2));
                                out[j][2 * k + r] = v;
                            }
                    if (active) write_group<kNP>(a, si, si.row0 + t0 + t, cfirst, nc, part, b > 0, out);
                }
            }
        }
    }
}

template <int NT, int OB, int MINB, int CB>
__global__ void __launch_bounds__(NT, MINB) degridder_oct_kernel(KernelArgs a) {
    degridder_oct_body<NT, OB, CB>(a);
}

template <int NT, int OB, int MINB, int CB>
cudaError_t launch_oct(const KernelArgs &a, cudaStream_t stream) {
    if (a.S % 2 != 0) return cudaErrorInvalidValue;
    void (*kern)(KernelArgs) = degridder_oct_kernel<NT, OB, MINB, CB>;
    const size_t smem = oct_layout(a.S, a.C, OB).total;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    if (a.share_den > 1) blocks = blocks / a.share_den > 0 ? blocks / a.share_den : 1;
    if (a.max_ctas > 0 && blocks > a.max_ctas) blocks = a.max_ctas;
    if (blocks > a.nr_subgrids) blocks = a.nr_subgrids;
    kern<<<(unsigned)blocks, NT, smem, stream>>>(a);
    return cudaGetLastError();
}

template <int NT, int QB, int MINB, int CB, int UNR, bool KSM = false, bool COL = false, int RUN = 0, bool PF = false,
          int MAXR = 0>
cudaError_t launch_quad(const KernelArgs &a, cudaStream_t stream) {
    if (a.S % 2 != 0) return cudaErrorInvalidValue;
    void (*kern)(KernelArgs);
    if constexpr (MAXR > 0)
        kern = degridder_quad_kernel_r<MAXR, NT, QB, CB, UNR, KSM, COL, RUN, PF>;
    else
        kern = degridder_quad_kernel<NT, QB, MINB, CB, UNR, KSM, COL, RUN, PF>;
    const size_t smem = quad_layout(a.S, a.C, QB).total;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    if (a.share_den > 1) blocks = blocks / a.share_den > 0 ? blocks / a.share_den : 1;
    if (a.max_ctas > 0 && blocks > a.max_ctas) blocks = a.max_ctas;
    if (blocks > a.nr_subgrids) blocks = a.nr_subgrids;
    kern<<<(unsigned)blocks, NT, smem, stream>>>(a);
    return cudaGetLastError();
}

} // namespace

int degridder_cp_shapes() { return 25; }

// Channel-pair shapes (index within this family):
//   0: 128 threads, 8-channel groups, 256-pixel batches, 4 CTAs/SM (16 warps)
//   1: 128 threads, 8-channel groups, 3 CTAs/SM, pixel loop unrolled by two
//   2: 128 threads, 16-channel groups, 2 CTAs/SM
//   3: 128 threads, 8-channel groups, Gauss MACs, 3 CTAs/SM
//   4: 256 threads, 8-channel groups, 2 CTAs/SM (16 warps)
//   5: 128 threads, 16-channel groups, Gauss MACs, 2 CTAs/SM
//   6: 128 threads, 8-channel groups, Gauss MACs, 2 CTAs/SM (registers uncapped)
//   7: shape 6 with the pixel loop unrolled by two
//   8: 128 threads, 8-channel groups, 2 CTAs/SM, pixel loop unrolled by two
//   9: shape 6 with the pixel loop unrolled by four
//  10: shape 7 with 256-pixel batches
//  11: shape 8 with the pixel loop unrolled by four
//  12: shape 6 with the pixel loop unrolled by eight
//  13: mirror quads, 128 threads, 8-channel groups, 256-quad batches, 2 CTAs/SM
//  14: mirror quads, 128 threads, 8-channel groups, 256-quad batches, 3 CTAs/SM (12 warps)
//  15: shape 13 with the quad loop unrolled by two
//  16: shape 14 reading each channel pair's kappa from shared memory when used
//  17: mirror quads in column form (P kept per column run), 2 CTAs/SM
//  18: shape 17 with the phasors of all channel pairs formed first
//  19: shape 17 with runs of 4 quads as straight-line blocks (S = 32)
//  20: shapes 18 and 19 together
//  21: column form, 96 threads x 3 CTAs/SM (9 warps), 128-quad batches
//  22: shape 21 with the phasors first
//  23: shape 17 with runs of 8 quads (S = 64)
//  24: swap-symmetric octets, 128 threads, 8-channel groups, 128-octet batches, 2 CTAs/SM
cudaError_t launch_degridder_cp(const KernelArgs &a, cudaStream_t stream, int shape) {
    switch (shape) {
    case 18: return launch_quad<128, 256, 2, 8, 1, true, true, 0, true>(a, stream);
    case 19: return launch_quad<128, 256, 2, 8, 1, true, true, 4>(a, stream);
    case 20: return launch_quad<128, 256, 2, 8, 1, true, true, 4, true>(a, stream);
    case 21: return launch_quad<96, 128, 3, 8, 1, true, true, 0, false, 224>(a, stream);
    case 22: return launch_quad<96, 128, 3, 8, 1, true, true, 0, true, 224>(a, stream);
    case 23: return launch_quad<128, 256, 2, 8, 1, true, true, 8>(a, stream);
    case 24: return launch_oct<128, 128, 2, 8>(a, stream);
    case 13: return launch_quad<128, 256, 2, 8, 1>(a, stream);
    case 14: return launch_quad<128, 256, 3, 8, 1>(a, stream);
    case 15: return launch_quad<128, 256, 2, 8, 2>(a, stream);
    case 16: return launch_quad<128, 256, 3, 8, 1, true>(a, stream);
    case 17: return launch_quad<128, 256, 2, 8, 1, true, true>(a, stream);
    case 1: return launch_cp<128, 512, 3, 8, 0, 2>(a, stream);
    case 2: return launch_cp<128, 512, 2, 16, 0, 1>(a, stream);
    case 3: return launch_cp<128, 512, 3, 8, kGaussCp, 1>(a, stream);
    case 4: return launch_cp<256, 512, 2, 8, 0, 1>(a, stream);
    case 5: return launch_cp<128, 512, 2, 16, kGaussCp, 1>(a, stream);
    case 6: return launch_cp<128, 512, 2, 8, kGaussCp, 1>(a, stream);
    case 7: return launch_cp<128, 512, 2, 8, kGaussCp, 2>(a, stream);
    case 8: return launch_cp<128, 512, 2, 8, 0, 2>(a, stream);
    case 9: return launch_cp<128, 512, 2, 8, kGaussCp, 4>(a, stream);
    case 10: return launch_cp<128, 256, 2, 8, kGaussCp, 2>(a, stream);
    case 11: return launch_cp<128, 512, 2, 8, 0, 4>(a, stream);
    case 12: return launch_cp<128, 512, 2, 8, kGaussCp, 8>(a, stream);
    default: return launch_cp<128, 256, 4, 8, 0, 1>(a, stream);
    }
}

} // namespace idg
