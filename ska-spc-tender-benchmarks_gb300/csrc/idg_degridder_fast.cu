// idg_degridder_fast.cu -- the batched degridder: persistent CTAs, packed
// FP32x2 pixel pairs, warp-shuffle combination of partial visibilities.
//
// Same result as the plain degridder (idg_degridder.cu):
//   V[t][c] = sum_pixels P'(x, y) exp(-i phase),  P' = A(taper * subgrid).
// Work decomposition:
//  * A CTA of 128 threads stages the subgrid's prepared pixels (A-term and
//    taper applied) in shared memory as pixel PAIRS laid out for packed
//    arithmetic: per pair and correlation (re_a, re_b, im_a, im_b) and
//    (-re_a, -re_b); the pair's geometry (hx, hy, n) is staged once per CTA.
//  * A visibility group is one timestep x CB channels (CB = 4 or 8).  Four
//    lanes share a group, each summing a quarter of the pixel pairs; a lane
//    keeps the group's CB x 4 complex partial sums as packed pairs (one half
//    per pixel of the pair) and so issues two fma.rn.f32x2 per complex MAC of
//    two pixels (or, in the Gauss variant, three per two complex MACs).
//  * At the end of a group the two halves are added and the four lanes'
//    partial sums are combined with warp shuffles; each lane writes CB/4
//    channels.
//  * Phase handling is the gridder's (idg_gridder_fast.cu): FP64 per-tile
//    coefficients, tau0 reduced to [-pi, pi] per (pair, timestep), and the
//    per-channel sincos unreduced when the tile's bound allows.
#include "idg_device.cuh"
#include "idg_internal.h"
#include "idg_ptx.cuh"

namespace idg {

namespace {

constexpr int kMaxCB = 8;               // channels per visibility group, at most (template CB = 4 or 8)
constexpr int kLanesPerGroup = 4;
constexpr int kGroupsPerWarp = 32 / kLanesPerGroup;
constexpr int kTimeTile = 64;
constexpr float kFastBound = 48.f;

constexpr float kInv2Pi = 0.159154943091895335769f;
constexpr float k2PiHi = 6.28125f;
constexpr float k2PiLo = 1.9353071795864769253e-3f;

struct Head {
    int next, fast, qmax_bits, kmax_bits;
};

struct Layout {
    size_t pix, geo, coef, kappa, total;
};

__host__ __device__ inline Layout layout(int S, int C, int batch_pairs) {
    Layout L;
    size_t off = 64;
    L.pix = off;   off += (size_t)batch_pairs * 96;          // 4 x (re_a,re_b,im_a,im_b) + 2 x (-re pairs)
    L.geo = off;   off += (size_t)(S * S / 2) * 24;          // (hx_a,hx_b) (hy,hy) (n_a,n_b)
    L.coef = off;  off += (size_t)kTimeTile * 48;            // (a,a,b,b) (g,g,qu,qu) (qv,qv,qw,qw)
    L.kappa = off; off += (size_t)(C + kMaxCB) * 4;          // kappa per channel, padded with zeros
    L.total = (off + 15) & ~size_t(15);
    return L;
}

__device__ __forceinline__ f2 reduce_2pi(f2 x) {
    const f2 M = pack2(12582912.0f, 12582912.0f);
    f2 k = fmul2(x, pack2(kInv2Pi, kInv2Pi));
    k = fsub2(fadd2(k, M), M);
    x = ffma2(k, pack2(-k2PiHi, -k2PiHi), x);
    return ffma2(k, pack2(-k2PiLo, -k2PiLo), x);
}

template <bool FTZ>
__device__ __forceinline__ void sincos_pair(f2 x, f2 &c, f2 &s) {
    float x0, x1, s0, c0, s1, c1;
    unpack2(x, x0, x1);
    if (FTZ) {
        s0 = sin_ftz(x0);
        c0 = cos_ftz(x0);
        s1 = sin_ftz(x1);
        c1 = cos_ftz(x1);
    } else {
        __sincosf(x0, &s0, &c0);
        __sincosf(x1, &s1, &c1);
    }
    c = pack2(c0, c1);
    s = pack2(s0, s1);
}

// Kernel variant bits (the FLAGS template argument).
constexpr int kFtz = 2;    // SFU sine/cosine flushing subnormal arguments
constexpr int kGauss = 4;  // three-multiplication MACs (12 accumulators per channel)
constexpr int kUnroll2 = 8; // pixel-pair loop unrolled by two

// Partial visibilities of one pixel pair for the group's channels (four complex
// MACs per correlation):  V += P (cos - i sin).
template <int kCB, bool FAST, bool FTZ>
__device__ __forceinline__ void pair_macs(f2 (&acc)[kCB][8], const f2 (&kc)[kCB], f2 tau0, f2 Q, const float4 *d) {
    const float4 e0 = d[0], e1 = d[1], e2 = d[2], e3 = d[3], e4 = d[4], e5 = d[5];
    const f2 pr0 = pack2(e0.x, e0.y), pi0 = pack2(e0.z, e0.w);
    const f2 pr1 = pack2(e1.x, e1.y), pi1 = pack2(e1.z, e1.w);
    const f2 pr2 = pack2(e2.x, e2.y), pi2 = pack2(e2.z, e2.w);
    const f2 pr3 = pack2(e3.x, e3.y), pi3 = pack2(e3.z, e3.w);
    const f2 nr0 = pack2(e4.x, e4.y), nr1 = pack2(e4.z, e4.w);
    const f2 nr2 = pack2(e5.x, e5.y), nr3 = pack2(e5.z, e5.w);
#pragma unroll
    for (int j = 0; j < kCB; ++j) {
        f2 x = ffma2(kc[j], Q, tau0);
        if (!FAST) x = reduce_2pi(x);
        f2 C, Sn;
        sincos_pair<FTZ>(x, C, Sn);
        // re += pr c + pi s ; im += pi c - pr s
        acc[j][0] = ffma2(pi0, Sn, ffma2(pr0, C, acc[j][0]));
        acc[j][1] = ffma2(nr0, Sn, ffma2(pi0, C, acc[j][1]));
        acc[j][2] = ffma2(pi1, Sn, ffma2(pr1, C, acc[j][2]));
        acc[j][3] = ffma2(nr1, Sn, ffma2(pi1, C, acc[j][3]));
        acc[j][4] = ffma2(pi2, Sn, ffma2(pr2, C, acc[j][4]));
        acc[j][5] = ffma2(nr2, Sn, ffma2(pi2, C, acc[j][5]));
        acc[j][6] = ffma2(pi3, Sn, ffma2(pr3, C, acc[j][6]));
        acc[j][7] = ffma2(nr3, Sn, ffma2(pi3, C, acc[j][7]));
    }
}

// Gauss form of pair_macs: with the pixel a + ib and the phasor c + id =
// cos - i sin, k1 = a (c + d) = a (cos - sin), -k2 = (a + b) sin,
// k3 = (b - a) cos; Re = k1 + (-k2), Im = k1 + k3.  The staged operands per
// correlation are the pixel-pair vectors a, a + b, b - a.
template <int kCB, bool FAST, bool FTZ>
__device__ __forceinline__ void pair_macs(f2 (&acc)[kCB][12], const f2 (&kc)[kCB], f2 tau0, f2 Q, const float4 *d) {
    const uint32_t base = smem_addr(d);
    f2 o[12];
#pragma unroll
    for (int q = 0; q < 6; ++q) lds2(base + 16 * q, o[2 * q], o[2 * q + 1]);
#pragma unroll
    for (int j = 0; j < kCB; ++j) {
        f2 x = ffma2(kc[j], Q, tau0);
        if (!FAST) x = reduce_2pi(x);
        f2 C, Sn;
        sincos_pair<FTZ>(x, C, Sn);
        const f2 cms = fsub2(C, Sn);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            acc[j][3 * k] = ffma2(o[3 * k], cms, acc[j][3 * k]);
            acc[j][3 * k + 1] = ffma2(o[3 * k + 1], Sn, acc[j][3 * k + 1]);
            acc[j][3 * k + 2] = ffma2(o[3 * k + 2], C, acc[j][3 * k + 2]);
        }
    }
}

// One lane's share of a visibility group: pixel pairs part, part + 4, ... of
// the staged batch (the 4 lanes of a group split the batch).  The FAST/slow
// phase path is chosen once per group, outside the pixel loop.
template <int kCB, bool FAST, int FLAGS, int NACC>
__device__ __forceinline__ void group_pixels(f2 (&acc)[kCB][NACC], const f2 (&kc)[kCB], f2 A2, f2 B2, f2 G2, f2 QU,
                                             f2 QV, f2 QW, const f2 *geo, const float4 *pix, int pb, int part, int np) {
    constexpr bool FTZ = (FLAGS & kFtz) != 0;
#pragma unroll((FLAGS & kUnroll2) ? 2 : 1)
    for (int i = part; i < np; i += kLanesPerGroup) {
        const int p = pb + i;
        const f2 hx = geo[3 * p], hy = geo[3 * p + 1], nn = geo[3 * p + 2];
        const f2 tau0 = reduce_2pi(ffma2(A2, hx, ffma2(B2, hy, fmul2(G2, nn))));
        const f2 Q = ffma2(QU, hx, ffma2(QV, hy, fmul2(QW, nn)));
        pair_macs<kCB, FAST, FTZ>(acc, kc, tau0, Q, pix + 6 * i);
    }
}

// Kernel shape: NT threads per CTA, BATCH pixel pairs staged per pass, at least
// MINB CTAs per SM (register cap), CB channels per visibility group (the
// per-(pixel pair, timestep) phase terms are computed once per group, so a
// larger group amortises them further); FLAGS: kFtz, kGauss.
template <int NT, int BATCH, int MINB, int FLAGS, int CB>
__global__ void __launch_bounds__(NT, MINB) degridder_fast_kernel(KernelArgs a) {
    constexpr int kT = NT, kBatchPairs = BATCH, kCB = CB;
    static_assert(CB == 4 || CB == 8, "channel groups of 4 or 8");
    constexpr bool FTZ = (FLAGS & kFtz) != 0, kG = (FLAGS & kGauss) != 0;
    constexpr int kAcc = kG ? 12 : 8;
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = a.S, S2 = S * S, npairs = S2 / 2;
    const Layout L = layout(S, a.C, BATCH);
    Head *head = reinterpret_cast<Head *>(smem);
    float4 *pix = reinterpret_cast<float4 *>(smem + L.pix);
    f2 *geo = reinterpret_cast<f2 *>(smem + L.geo);
    float4 *coef = reinterpret_cast<float4 *>(smem + L.coef);
    float *kap = reinterpret_cast<float *>(smem + L.kappa);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gw = lane / kLanesPerGroup, part = lane % kLanesPerGroup;
    const bool refcpu = (a.flags & IDG_FLAG_DEGRID_ATERM_REFCPU) != 0;
    const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;

    for (int p = tid; p < npairs; p += kT) {
        const float3 g0 = pixel_geometry(2 * p, S, a.image_size);
        const float3 g1 = pixel_geometry(2 * p + 1, S, a.image_size);
        geo[3 * p + 0] = pack2(g0.x, g1.x);
        geo[3 * p + 1] = pack2(g0.y, g1.y);
        geo[3 * p + 2] = pack2(g0.z, g1.z);
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

        for (int pb = 0; pb < npairs; pb += kBatchPairs) {
            const int np = min(kBatchPairs, npairs - pb);
            __syncthreads(); // previous batch consumed
            // ---- stage prepared pixel pairs
            for (int i = tid; i < np; i += kT) {
                const int p = pb + i;
                cf v[2][4];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int q = 2 * p + h;
                    const float sph = taper ? a.taper[q] : 1.f;
#pragma unroll
                    for (int pol = 0; pol < 4; ++pol) {
                        const float2 x = a.subgrids[((size_t)s * 4 + pol) * S2 + q];
                        v[h][pol] = {sph * x.x, sph * x.y};
                    }
                    cf j1[4], j2[4];
                    load_jones(a1 + 2 * q, j1);
                    load_jones(a2 + 2 * q, j2);
                    if (refcpu)
                        aterm_gridder(v[h], j1, j2);
                    else
                        aterm_adjoint(v[h], j1, j2);
                }
                float4 *d = pix + 6 * i;
                if (kG) {
                    // per correlation the pair vectors a, a + b, b - a
                    float e[12][2];
#pragma unroll
                    for (int pol = 0; pol < 4; ++pol)
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            e[3 * pol][h] = v[h][pol].re;
                            e[3 * pol + 1][h] = v[h][pol].re + v[h][pol].im;
                            e[3 * pol + 2][h] = v[h][pol].im - v[h][pol].re;
                        }
#pragma unroll
                    for (int q = 0; q < 6; ++q)
                        d[q] = make_float4(e[2 * q][0], e[2 * q][1], e[2 * q + 1][0], e[2 * q + 1][1]);
                } else {
#pragma unroll
                    for (int pol = 0; pol < 4; ++pol)
                        d[pol] = make_float4(v[0][pol].re, v[1][pol].re, v[0][pol].im, v[1][pol].im);
                    d[4] = make_float4(-v[0][0].re, -v[1][0].re, -v[0][1].re, -v[1][1].re);
                    d[5] = make_float4(-v[0][2].re, -v[1][2].re, -v[0][3].re, -v[1][3].re);
                }
            }

            for (int t0 = 0; t0 < si.T; t0 += kTimeTile) {
                const int tt = min(kTimeTile, si.T - t0);
                __syncthreads();
                for (int t = tid; t < tt; t += kT) {
                    const float *p = a.uvw + 3 * ((int64_t)si.row0 + t0 + t);
                    const double u = p[0], v = p[1], w = p[2];
                    double ca = ((double)si.X + S * 0.5 - a.G * 0.5) / S - kref * u * d2pi;
                    double cbv = ((double)si.Y + S * 0.5 - a.G * 0.5) / S - kref * v * d2pi;
                    ca -= 2.0 * rint(ca * 0.5);
                    cbv -= 2.0 * rint(cbv * 0.5);
                    const double cg = kTwoPi * (double)a.w_step * ((double)si.Z + 0.5) - kref * w;
                    const float A = (float)(kTwoPi * ca), B = (float)(kTwoPi * cbv), Gv = (float)cg;
                    const float qu = (float)(-u * d2pi * kTwoPi), qv = (float)(-v * d2pi * kTwoPi), qw = (float)(-w);
                    coef[3 * t + 0] = make_float4(A, A, B, B);
                    coef[3 * t + 1] = make_float4(Gv, Gv, qu, qu);
                    coef[3 * t + 2] = make_float4(qv, qv, qw, qw);
                    atomicMax(&head->qmax_bits, __float_as_int(fabsf(qu) * hmax + fabsf(qv) * hmax + fabsf(qw) * nmax));
                }
                __syncthreads();
                if (tid == 0) {
                    head->fast = (3.1416f + __int_as_float(head->kmax_bits) * __int_as_float(head->qmax_bits)) <= kFastBound;
                    head->qmax_bits = 0;
                }
                __syncthreads();
                const bool fast = head->fast != 0;

                const int ngroups = tt * ncb;
                for (int gbase = warp * kGroupsPerWarp; gbase < ngroups; gbase += (kT / 32) * kGroupsPerWarp) {
                    const int grp = gbase + gw;
                    const bool active = grp < ngroups;
                    const int gg = active ? grp : 0;
                    const int t = gg / ncb, cfirst = (gg - t * ncb) * kCB;
                    const float4 c0 = coef[3 * t], c1 = coef[3 * t + 1], c2 = coef[3 * t + 2];
                    const f2 A2 = pack2(c0.x, c0.y), B2 = pack2(c0.z, c0.w), G2 = pack2(c1.x, c1.y);
                    const f2 QU = pack2(c1.z, c1.w), QV = pack2(c2.x, c2.y), QW = pack2(c2.z, c2.w);
                    f2 kc[kCB];
#pragma unroll
                    for (int j = 0; j < kCB; ++j) {
                        const float kv = kap[cfirst + j];
                        kc[j] = pack2(kv, kv);
                    }
                    f2 acc[kCB][kAcc];
#pragma unroll
                    for (int j = 0; j < kCB; ++j)
#pragma unroll
                        for (int r = 0; r < kAcc; ++r) acc[j][r] = 0ull;

                    if (fast)
                        group_pixels<kCB, true, FLAGS>(acc, kc, A2, B2, G2, QU, QV, QW, geo, pix, pb, part, np);
                    else
                        group_pixels<kCB, false, FLAGS>(acc, kc, A2, B2, G2, QU, QV, QW, geo, pix, pb, part, np);
                    // fold the pair halves, then combine the four lanes of the group
                    float vsum[kCB][8];
#pragma unroll
                    for (int j = 0; j < kCB; ++j)
#pragma unroll
                        for (int r = 0; r < 8; ++r) {
                            float lo, hi;
                            if (kG) // Re = k1 + (-k2), Im = k1 + k3
                                unpack2(fadd2(acc[j][3 * (r / 2)], acc[j][3 * (r / 2) + 1 + (r & 1)]), lo, hi);
                            else
                                unpack2(acc[j][r], lo, hi);
                            float v = lo + hi;
                            v += __shfl_xor_sync(0xffffffffu, v, 1);
                            v += __shfl_xor_sync(0xffffffffu, v, 2);
                            vsum[j][r] = v;
                        }
                    if (active) {
                        float4 *row = a.vis + ((int64_t)si.row0 + t0 + t) * a.C * 2;
#pragma unroll
                        for (int j = 0; j < kCB; ++j) {
                            if (j % kLanesPerGroup != part || cfirst + j >= nc) continue;
                            const int c = si.c0 + cfirst + j;
                            float4 va = make_float4(vsum[j][0], vsum[j][1], vsum[j][2], vsum[j][3]);
                            float4 vb = make_float4(vsum[j][4], vsum[j][5], vsum[j][6], vsum[j][7]);
                            if (pb > 0) {
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
}

template <int NT, int BATCH, int MINB, int FLAGS = 0, int CB = 4>
cudaError_t launch_shape(const KernelArgs &a, cudaStream_t stream) {
    auto kern = degridder_fast_kernel<NT, BATCH, MINB, FLAGS, CB>;
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

} // namespace

// Launch shapes of the batched degridder (index = shape id).
// Shapes 0-14 are the pixel-pair kernel above; 15 and up the channel-pair kernel.
int degridder_fast_shapes() { return 15 + degridder_cp_shapes(); }

cudaError_t launch_degridder_fast(const KernelArgs &a, cudaStream_t stream, int shape) {
    if (shape >= 15) return launch_degridder_cp(a, stream, shape - 15);
    switch (shape) {
    case 1: return launch_shape<128, 512, 4>(a, stream); // 16 warps/SM, register cap 128
    case 2: return launch_shape<256, 512, 2>(a, stream); // 16 warps/SM in 256-thread CTAs
    case 3: return launch_shape<128, 256, 4>(a, stream); // smaller staging batches
    case 4: return launch_shape<128, 512, 2>(a, stream); // 8 warps/SM, registers uncapped
    case 5: return launch_shape<128, 512, 2, kFtz>(a, stream); // shape 4, subnormal-flushing SFU sin/cos
    case 6: return launch_shape<128, 512, 3, kFtz>(a, stream); // shape 0, subnormal-flushing SFU sin/cos
    case 7: return launch_shape<128, 512, 2, kGauss>(a, stream); // shape 4 with Gauss MACs
    case 8: return launch_shape<128, 512, 3, kGauss>(a, stream); // shape 0 with Gauss MACs
    case 9: return launch_shape<256, 512, 1, kGauss>(a, stream); // 8 warps/SM in 256-thread CTAs, Gauss MACs
    case 10: return launch_shape<128, 512, 2, 0, 8>(a, stream); // shape 4 with 8-channel groups
    case 11: return launch_shape<128, 512, 2, kGauss, 8>(a, stream); // shape 7 with 8-channel groups
    case 12: return launch_shape<256, 512, 1, kGauss, 8>(a, stream); // shape 9 with 8-channel groups
    case 13: return launch_shape<128, 512, 2, kUnroll2>(a, stream); // shape 4, pixel loop unrolled by two
    case 14: return launch_shape<128, 512, 2, kUnroll2, 8>(a, stream); // shape 10, pixel loop unrolled by two
    default: return launch_shape<128, 512, 3>(a, stream); // 12 warps/SM
    }
}

} // namespace idg
