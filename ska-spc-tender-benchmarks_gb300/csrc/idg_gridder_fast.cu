// idg_gridder_fast.cu -- the batched gridder: persistent CTAs, TMA-staged
// visibilities, packed-FP32 pixel pairs.
//
// Same result as the plain gridder (idg_gridder.cu): subgrid = taper * A1^H P A2
// with P = sum_{t,c} V[t][c] exp(i phase), phase carried with FP64 per-subgrid
// offsets.  Differences in how the work is done:
//  * CTAs are persistent and pull subgrids from a global counter (optionally
//    through a cost-sorted work list), so uneven subgrids balance in one launch.
//  * Each thread owns 4 pixel PAIRS (8 pixels, two adjacent x per pair) and
//    keeps their accumulators as packed FP32x2 registers: every complex MAC of
//    a pixel pair is two fma.rn.f32x2, halving issue slots per pixel-visibility
//    (17 FMA of work issue as ~9 instructions).
//  * A tile of visibilities is copied global -> shared with cp.async.bulk (one
//    bulk copy per row, completion counted on an mbarrier, bounded wait) and
//    expanded once per tile into the operand pairs the packed MACs read as
//    warp-wide broadcasts: (re,re), (im,im), (-im,-im) per correlation.
//  * The phase is kept in radians: per (pixel pair, timestep) the FP64-derived
//    offset part tau0 is reduced to [-pi, pi]; per channel x = tau0 + kappa*Q.
//    When a tile's bound pi + max|kappa| max|Q| stays below kFastBound the
//    sincos takes x directly (the SFU reduces the argument itself; the error
//    grows as |x| * 2^-24), otherwise x is reduced to [-pi, pi] first.
//  * Shapes 15-17 replace the per-channel sincos of those tiles by an
//    exact channel recurrence (grid_tile_recur): the autotuner keeps them
//    when they are faster on the data at hand.
#include "idg_device.cuh"
#include "idg_internal.h"
#include "idg_ptx.cuh"

namespace idg {

namespace {

constexpr int kMaxTT = 64;                    // timesteps per tile, at most
constexpr float kFastBound = 48.f;            // radians
constexpr uint64_t kWaitNs = 2000000000ull;   // a staged copy not complete after 2 s is declared lost

constexpr float kInv2Pi = 0.159154943091895335769f;
constexpr float k2PiHi = 6.28125f;                        // 2 pi split for exact k * 2pi_hi (k < 2^15)
constexpr float k2PiLo = 1.9353071795864769253e-3f;       // 2 pi - k2PiHi

struct SmemHead {
    uint64_t bar;
    int fast;        // tile uses the unreduced path
    int qmax_bits;   // max |Q| of the tile (float bits, non-negative)
    int kmax_bits;   // max |kappa| of the subgrid
    int abort;       // a staged copy did not arrive in time
    int next;        // work item
};

struct Layout {
    size_t raw, vexp, coef, kappa, chain, geo, total;
};

__host__ __device__ inline Layout layout(int S, int C, int tile_vis) {
    Layout L;
    size_t off = 64;                                   // SmemHead
    L.raw = off;  off += (size_t)tile_vis * 32;        // raw visibilities (TMA destination)
    L.vexp = off; off += (size_t)tile_vis * 96;        // expanded operand pairs
    L.coef = off; off += (size_t)kMaxTT * 48;          // per timestep: (a,a,b,b) (g,g,qu,qu) (qv,qv,qw,qw)
    L.kappa = off; off += (size_t)C * 8;               // (kappa, kappa)
    off = (off + 15) & ~size_t(15);
    L.chain = off; off += (size_t)C * 16;              // channel chains (recurrence form)
    L.geo = off;  off += (size_t)(S * S / 2) * 24;      // per pair: (hx0,hx1) (hy,hy) (n0,n1)
    L.total = off;
    return L;
}

// The mirror-quad kernel's own layout: raw and expanded visibilities (4
// duplicated operand pairs, 64 B, per visibility), coefficients and kappa; its
// quad geometry follows `total` (the pixel-pair geometry and channel chains
// of the layout above are not used).
struct QuadLayout {
    size_t raw, vexp, coef, kappa, total;
};
__host__ __device__ inline QuadLayout quad_layout(int C, int tile_vis) {
    QuadLayout L;
    size_t off = 64;                                   // SmemHead
    L.raw = off;  off += (size_t)tile_vis * 32;
    L.vexp = off; off += (size_t)tile_vis * 64;
    L.coef = off; off += (size_t)kMaxTT * 48;
    L.kappa = off; off += (size_t)C * 8;
    L.total = (off + 15) & ~size_t(15);
    return L;
}

__device__ __forceinline__ f2 dup(float v) { return pack2(v, v); }
__device__ __forceinline__ f2 neg2(f2 v) { return v ^ 0x8000000080000000ull; }

// Channel chain of the recurrence form: channels [c, c + len) of a subgrid
// whose consecutive wavenumber differences kappa[i+1] - kappa[i] (exact in
// float) all equal d.  `newd` is set when d differs from the previous chain's
// (or the chain opens a channel chunk), i.e. when the step factor must be
// recomputed.
struct ChainInfo {
    int len;
    float d;
    int newd;
    int pad;
};
constexpr int kMaxChain = 16; // channels per chain at most: the re-anchoring interval

// x - 2 pi rint(x / 2 pi), elementwise on a pair (Cody-Waite, two constants).
__device__ __forceinline__ f2 reduce_2pi(f2 x) {
    const f2 M = pack2(12582912.0f, 12582912.0f);
    f2 k = fmul2(x, pack2(kInv2Pi, kInv2Pi));
    k = fsub2(fadd2(k, M), M);
    x = ffma2(k, pack2(-k2PiHi, -k2PiHi), x);
    return ffma2(k, pack2(-k2PiLo, -k2PiLo), x);
}

// FTZ: the SFU instructions flushing subnormal arguments (sin/cos.approx.ftz)
// instead of __sincosf's default that honours them.
template <bool FTZ = false>
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

// Phasors of one channel for all pixel pairs of the thread.
template <int PAIRS, bool FAST, bool FTZ>
__device__ __forceinline__ void channel_phasors(f2 kc, const f2 (&tau0)[PAIRS], const f2 (&Q)[PAIRS], f2 (&C)[PAIRS],
                                                f2 (&Sn)[PAIRS]) {
#pragma unroll
    for (int j = 0; j < PAIRS; ++j) {
        f2 x = ffma2(kc, Q[j], tau0[j]);
        if (!FAST) x = reduce_2pi(x);
        sincos_pair<FTZ>(x, C[j], Sn[j]);
    }
}

// Three-multiplication complex MAC (Gauss): with V = a + ib and the phasor
// c + id,  k1 = a (c + d),  k2 = (a + b) d,  k3 = (b - a) c  give
// Re(V e) = k1 - k2 and Im(V e) = k1 + k3.  The three products are summed
// separately over all visibilities and combined once in the epilogue, so a
// pixel pair costs 12 fma.rn.f32x2 + 1 add.rn.f32x2 per visibility instead
// of 16.  Operands per visibility, pre-expanded per tile (duplicated into both
// halves): for each correlation (a, a), (a + b, a + b), (b - a, b - a).
template <int PAIRS>
__device__ __forceinline__ void channel_macs(f2 (&acc)[PAIRS][12], const float4 *vv, const f2 (&C)[PAIRS],
                                             const f2 (&Sn)[PAIRS]) {
    const uint32_t base = smem_addr(vv);
    f2 o[12];
#pragma unroll
    for (int q = 0; q < 6; ++q) lds2(base + 16 * q, o[2 * q], o[2 * q + 1]);
#pragma unroll
    for (int j = 0; j < PAIRS; ++j) {
        const f2 cpd = fadd2(C[j], Sn[j]);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            acc[j][3 * k] = ffma2(o[3 * k], cpd, acc[j][3 * k]);
            acc[j][3 * k + 1] = ffma2(o[3 * k + 1], Sn[j], acc[j][3 * k + 1]);
            acc[j][3 * k + 2] = ffma2(o[3 * k + 2], C[j], acc[j][3 * k + 2]);
        }
    }
}

// P += V * (cos + i sin) for every pixel pair: re += vr c - vi s ; im += vr s + vi c
template <int PAIRS>
__device__ __forceinline__ void channel_macs(f2 (&acc)[PAIRS][8], const float4 *vv, const f2 (&C)[PAIRS],
                                             const f2 (&Sn)[PAIRS]) {
    const float4 e0 = vv[0], e1 = vv[1], e2 = vv[2], e3 = vv[3], e4 = vv[4], e5 = vv[5];
    const f2 vr0 = pack2(e0.x, e0.y), vi0 = pack2(e0.z, e0.w);
    const f2 vr1 = pack2(e1.x, e1.y), vi1 = pack2(e1.z, e1.w);
    const f2 vr2 = pack2(e2.x, e2.y), vi2 = pack2(e2.z, e2.w);
    const f2 vr3 = pack2(e3.x, e3.y), vi3 = pack2(e3.z, e3.w);
    const f2 ni0 = pack2(e4.x, e4.y), ni1 = pack2(e4.z, e4.w);
    const f2 ni2 = pack2(e5.x, e5.y), ni3 = pack2(e5.z, e5.w);
#pragma unroll
    for (int j = 0; j < PAIRS; ++j) {
        acc[j][0] = ffma2(ni0, Sn[j], ffma2(vr0, C[j], acc[j][0]));
        acc[j][1] = ffma2(vi0, C[j], ffma2(vr0, Sn[j], acc[j][1]));
        acc[j][2] = ffma2(ni1, Sn[j], ffma2(vr1, C[j], acc[j][2]));
        acc[j][3] = ffma2(vi1, C[j], ffma2(vr1, Sn[j], acc[j][3]));
        acc[j][4] = ffma2(ni2, Sn[j], ffma2(vr2, C[j], acc[j][4]));
        acc[j][5] = ffma2(vi2, C[j], ffma2(vr2, Sn[j], acc[j][5]));
        acc[j][6] = ffma2(ni3, Sn[j], ffma2(vr3, C[j], acc[j][6]));
        acc[j][7] = ffma2(vi3, C[j], ffma2(vr3, Sn[j], acc[j][7]));
    }
}

// Kernel variant bits (the PIPE template argument).
constexpr int kPipe = 1;     // software-pipelined channel loop
constexpr int kFtz = 2;      // SFU sine/cosine flushing subnormal arguments
constexpr int kGauss = 4;    // three-multiplication MACs (12 accumulators per pair)
constexpr int kUnroll2 = 8;  // channel loop unrolled by two
constexpr int kUnroll4 = 16; // channel loop unrolled by four
constexpr int kRecur = 32;   // channel recurrence on tiles within the unreduced bound

// One staged tile: tt timesteps x ncc channels.
// PIPE & kPipe: the channel loop is software pipelined -- the sincos of channel
// c+1 is issued before the MACs of channel c, so a warp keeps SFU and FMA work
// in flight together (more registers).  Otherwise phasors then MACs per channel.
// NACC = 8 (four complex MACs) or 12 (Gauss form); UNR = channel-loop unrolling.
template <int PAIRS, bool FAST, int PIPE, int NACC, int UNR>
__device__ __forceinline__ void grid_tile(f2 (&acc)[PAIRS][NACC], const int (&pr)[PAIRS], const float4 *coef,
                                          const f2 *geo, const float4 *vexp, const f2 *kp, int tt, int ncc) {
    for (int t = 0; t < tt; ++t) {
        const float4 c0 = coef[3 * t], c1 = coef[3 * t + 1], c2 = coef[3 * t + 2];
        const f2 A2 = pack2(c0.x, c0.y), B2 = pack2(c0.z, c0.w), G2 = pack2(c1.x, c1.y);
        const f2 QU = pack2(c1.z, c1.w), QV = pack2(c2.x, c2.y), QW = pack2(c2.z, c2.w);
        f2 tau0[PAIRS], Q[PAIRS];
#pragma unroll
        for (int j = 0; j < PAIRS; ++j) {
            const f2 hx = geo[3 * pr[j]], hy = geo[3 * pr[j] + 1], nn = geo[3 * pr[j] + 2];
            tau0[j] = reduce_2pi(ffma2(A2, hx, ffma2(B2, hy, fmul2(G2, nn))));
            Q[j] = ffma2(QU, hx, ffma2(QV, hy, fmul2(QW, nn)));
        }
        const float4 *vt = vexp + (size_t)t * ncc * 6;
        constexpr bool FTZ = (PIPE & kFtz) != 0;
        if (PIPE & kPipe) {
            f2 Cn[PAIRS], Sn[PAIRS];
            channel_phasors<PAIRS, FAST, FTZ>(kp[0], tau0, Q, Cn, Sn);
#pragma unroll UNR
            for (int c = 0; c + 1 < ncc; ++c) {
                f2 C[PAIRS], S[PAIRS];
#pragma unroll
                for (int j = 0; j < PAIRS; ++j) {
                    C[j] = Cn[j];
                    S[j] = Sn[j];
                }
                channel_phasors<PAIRS, FAST, FTZ>(kp[c + 1], tau0, Q, Cn, Sn);
                channel_macs<PAIRS>(acc, vt + 6 * c, C, S);
            }
            channel_macs<PAIRS>(acc, vt + 6 * (ncc - 1), Cn, Sn);
        } else {
#pragma unroll UNR
            for (int c = 0; c < ncc; ++c) {
                f2 C[PAIRS], S[PAIRS];
                channel_phasors<PAIRS, FAST, FTZ>(kp[c], tau0, Q, C, S);
                channel_macs<PAIRS>(acc, vt + 6 * c, C, S);
            }
        }
    }
}

// Recurrence form of one staged tile (unreduced-bound tiles only, Gauss MACs).
// The phase of channel c is x_c = tau0 + kappa_c Q, so along a chain of
// channels whose wavenumbers step by the same d,
// exp(i x_{c+1}) = exp(i x_c) exp(i d Q).  Per (pixel, timestep, chain): one
// sincos for the anchor channel, and one for exp(i d Q) when d changed;
// every other channel costs a complex multiplication on the FMA pipe instead
// of a sincos on the SFU.  Float wavenumbers of linearly spaced channels step
// by one of two neighbouring floats, so narrow bands give long chains (16
// channels over 150-160 MHz: 11 + 5 channels, one step factor); chains are at
// most kMaxChain long, which bounds the accumulated rounding to a few units in
// the last place of the phase.
template <int PAIRS, int UNR, bool FTZ, bool AHEAD>
__device__ __forceinline__ void grid_tile_recur(f2 (&acc)[PAIRS][12], const int (&pr)[PAIRS], const float4 *coef,
                                                const f2 *geo, const float4 *vexp, const f2 *kp,
                                                const ChainInfo *chains, int tt, int ncc) {
    for (int t = 0; t < tt; ++t) {
        const float4 c0 = coef[3 * t], c1 = coef[3 * t + 1], c2 = coef[3 * t + 2];
        const f2 A2 = pack2(c0.x, c0.y), B2 = pack2(c0.z, c0.w), G2 = pack2(c1.x, c1.y);
        const f2 QU = pack2(c1.z, c1.w), QV = pack2(c2.x, c2.y), QW = pack2(c2.z, c2.w);
        const float4 *vt = vexp + (size_t)t * ncc * 6;
        f2 Dc[PAIRS], Ds[PAIRS], Dn[PAIRS];
        for (int cs = 0; cs < ncc;) {
            const ChainInfo ch = chains[cs];
            f2 Rc[PAIRS], Rs[PAIRS];
#pragma unroll
            for (int j = 0; j < PAIRS; ++j) {
                // tau0 and Q per chain (not kept live across the channel loop)
                const f2 hx = geo[3 * pr[j]], hy = geo[3 * pr[j] + 1], nn = geo[3 * pr[j] + 2];
                const f2 tau0 = reduce_2pi(ffma2(A2, hx, ffma2(B2, hy, fmul2(G2, nn))));
                const f2 Q = ffma2(QU, hx, ffma2(QV, hy, fmul2(QW, nn)));
                sincos_pair<FTZ>(ffma2(kp[cs], Q, tau0), Rc[j], Rs[j]);
                if (ch.newd) {
                    sincos_pair<FTZ>(fmul2(dup(ch.d), Q), Dc[j], Ds[j]);
                    Dn[j] = neg2(Ds[j]);
                }
            }
            const int ce = cs + ch.len;
#pragma unroll UNR
            for (int c = cs; c < ce; ++c) {
                if (AHEAD) {
                    // next channel's phasor first, so its two dependent FMA levels
                    // overlap this channel's MACs
                    f2 nc_[PAIRS], ns_[PAIRS];
#pragma unroll
                    for (int j = 0; j < PAIRS; ++j) {
                        nc_[j] = ffma2(Rc[j], Dc[j], fmul2(Rs[j], Dn[j]));
                        ns_[j] = ffma2(Rc[j], Ds[j], fmul2(Rs[j], Dc[j]));
                    }
                    channel_macs<PAIRS>(acc, vt + 6 * c, Rc, Rs);
#pragma unroll
                    for (int j = 0; j < PAIRS; ++j) {
                        Rc[j] = nc_[j];
                        Rs[j] = ns_[j];
                    }
                } else {
                    channel_macs<PAIRS>(acc, vt + 6 * c, Rc, Rs);
#pragma unroll
                    for (int j = 0; j < PAIRS; ++j) {
                        const f2 rc = ffma2(Rc[j], Dc[j], fmul2(Rs[j], Dn[j]));
                        const f2 rs = ffma2(Rc[j], Ds[j], fmul2(Rs[j], Dc[j]));
                        Rc[j] = rc;
                        Rs[j] = rs;
                    }
                }
            }
            cs = ce;
        }
    }
}

// Chains of a subgrid's channels (one thread): maximal runs of equal
// wavenumber steps, cut at every channel chunk and after max_len channels
// (max_len <= kMaxChain).
__device__ inline void build_chains(const f2 *kap, ChainInfo *chains, int nc, int chunk, int max_len) {
    float hi, dprev = 0.f;
    int c = 0;
    while (c < nc) {
        const int cs = c;
        const int lim = min(min(nc, (cs / chunk + 1) * chunk), cs + max_len);
        const bool opens_chunk = cs % chunk == 0;
        float kprev, d = dprev;
        unpack2(kap[c], kprev, hi);
        ++c;
        if (c < lim) {
            float kc;
            unpack2(kap[c], kc, hi);
            d = kc - kprev;
            for (++c; c < lim; ++c) {
                kprev = kc;
                unpack2(kap[c], kc, hi);
                if (kc - kprev != d) break;
            }
        }
        // a one-channel chain never steps: it keeps the previous factor
        const bool newd = opens_chunk || (c - cs > 1 && __float_as_int(d) != __float_as_int(dprev));
        if (c - cs == 1 && opens_chunk) d = 0.f;
        chains[cs] = ChainInfo{c - cs, d, newd ? 1 : 0, 0};
        dprev = d;
    }
}

// One staged tile of a batched gridder.  Thread 0 issues one bulk copy per
// row (tt rows x ncc visibilities from channel c0 + cb) onto the mbarrier;
// meanwhile all threads compute the per-timestep phase coefficients (FP64,
// offsets reduced, stored as float pairs) and fold the tile's phase-slope
// bound into head->qmax_bits: the sum of the three slopes (QSUM, one phase
// per pixel) or their maximum (the factored forms, one argument per factor).
// Then the bounded wait.  Returns false when the copies did not arrive: the
// abort flag and the status bit are set, and the CTA must stop.
template <int NT, bool QSUM>
__device__ __forceinline__ bool stage_tile(const KernelArgs &a, const SubgridInfo &si, SmemHead *head, float4 *raw,
                                           float4 *coef, int t0, int tt, int cb, int ncc, double kref, double d2pi,
                                           float hmax, float nmax, uint32_t &phase) {
    const int tid = threadIdx.x, S = a.S;
    __syncthreads(); // previous tile fully consumed (raw, expanded operands, coef)
    if (tid == 0) {
        const uint32_t row_bytes = (uint32_t)ncc * 32u;
        // IDG_FLAG_TEST_LOST_COPY: expect 16 bytes that never come, so that the wait runs out
        const uint32_t lost = (a.flags & IDG_FLAG_TEST_LOST_COPY) ? 16u : 0u;
        fence_proxy_async();
        mbar_arrive_expect_tx(&head->bar, row_bytes * (uint32_t)tt + lost);
        const float4 *src = a.vis + ((int64_t)si.row0 + t0) * a.C * 2 + (int64_t)(si.c0 + cb) * 2;
        for (int r = 0; r < tt; ++r)
            bulk_g2s(raw + (size_t)r * ncc * 2, src + (int64_t)r * a.C * 2, row_bytes, &head->bar);
    }
    for (int t = tid; t < tt; t += NT) {
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
        const float qm = QSUM ? fabsf(qu) * hmax + fabsf(qv) * hmax + fabsf(qw) * nmax
                              : fmaxf(fmaxf(fabsf(qu) * hmax, fabsf(qv) * hmax), fabsf(qw) * nmax);
        atomicMax(&head->qmax_bits, __float_as_int(qm));
    }
    if (!mbar_wait_bounded(&head->bar, phase, kWaitNs)) {
        head->abort = 1;
        flag_status(a.status, kStatusTimeout);
    }
    __syncthreads();
    if (head->abort) {
        // give the copies in flight one more bounded wait before the CTA exits
        if (tid == 0) mbar_wait_bounded(&head->bar, phase, kWaitNs);
        return false;
    }
    phase ^= 1u;
    return true;
}

// Kernel shape: NT threads per CTA, PAIRS pixel pairs per thread per pass,
// TV visibilities per staged tile, at least MINB CTAs per SM (register cap).
template <int NT, int PAIRS, int TV, int MINB, int PIPE>
__global__ void __launch_bounds__(NT, MINB) gridder_fast_kernel(KernelArgs a) {
    constexpr int kT = NT, kPairs = PAIRS, kPassPairs = NT * PAIRS, kTileVis = TV, kMaxChunk = TV;
    constexpr bool kG = (PIPE & kGauss) != 0;
    constexpr int kAcc = kG ? 12 : 8, kUnr = (PIPE & kUnroll4) ? 4 : (PIPE & kUnroll2) ? 2 : 1;
    constexpr bool kRec = kG && (PIPE & kRecur) != 0;
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = a.S, S2 = S * S, npairs = S2 / 2;
    const Layout L = layout(S, a.C, TV);
    SmemHead *head = reinterpret_cast<SmemHead *>(smem);
    float4 *raw = reinterpret_cast<float4 *>(smem + L.raw);
    float4 *vexp = reinterpret_cast<float4 *>(smem + L.vexp);
    float4 *coef = reinterpret_cast<float4 *>(smem + L.coef);
    f2 *kap = reinterpret_cast<f2 *>(smem + L.kappa);
    f2 *geo = reinterpret_cast<f2 *>(smem + L.geo);
    ChainInfo *chains = reinterpret_cast<ChainInfo *>(smem + L.chain);
    const int tid = threadIdx.x;

    if (tid == 0) {
        mbar_init(&head->bar, 1);
        mbar_init_fence();
        head->abort = 0;
    }
    // pixel geometry of every pair, once per CTA (FP64 n as in math.hpp:31-37)
    for (int p = tid; p < npairs; p += kT) {
        const float3 g0 = pixel_geometry(2 * p, S, a.image_size);
        const float3 g1 = pixel_geometry(2 * p + 1, S, a.image_size);
        geo[3 * p + 0] = pack2(g0.x, g1.x);
        geo[3 * p + 1] = pack2(g0.y, g1.y);
        geo[3 * p + 2] = pack2(g0.z, g1.z);
    }
    __syncthreads();
    uint32_t phase = 0;
    const double d2pi = (double)a.image_size / (double)S / kTwoPi;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            head->next = atomicAdd(a.work_counter, 1);
            head->kmax_bits = 0;
            head->qmax_bits = 0;
        }
        __syncthreads();
        const int idx = head->next;
        if (idx >= a.nr_subgrids || head->abort) break;
        const int s = a.work_list ? a.work_list[idx] : idx;
        const SubgridInfo si = load_subgrid(a, s);
        const int nc = si.c1 - si.c0;
        if (!si.ok) {
            if (tid == 0) flag_status(a.status, kStatusBadPlan);
            for (int i = tid; i < 4 * S2; i += kT) a.subgrids[(size_t)s * 4 * S2 + i] = make_float2(0.f, 0.f);
            continue;
        }
        // channel offsets relative to the middle channel; max |kappa|
        const int cref = si.c0 + (nc > 0 ? (nc - 1) / 2 : 0);
        const double kref = nc > 0 ? (double)a.wavenumbers[cref] : 0.0;
        float kmax = 0.f;
        for (int c = tid; c < nc; c += kT) {
            const float kv = (float)((double)a.wavenumbers[si.c0 + c] - kref);
            kap[c] = dup(kv);
            kmax = fmaxf(kmax, fabsf(kv));
        }
        // block max of kmax through the head word (non-negative floats order as ints)
        if (kmax > 0.f) atomicMax(&head->kmax_bits, __float_as_int(kmax));
        __syncthreads();
        const float kappa_max = __int_as_float(head->kmax_bits);

        const int chunk = nc < kMaxChunk ? nc : kMaxChunk;
        const int TT = nc > 0 ? min(kMaxTT, kTileVis / chunk) : 1;
        // read after the staging barrier of the first tile
        if (kRec && tid == 0) build_chains(kap, chains, nc, chunk, kMaxChain);
        const float hmax = 0.5f * (float)(S - 1);
        const float3 gc = pixel_geometry(0, S, a.image_size);
        const float nmax = gc.z;

        for (int pass = 0; pass * kPassPairs < npairs; ++pass) {
            f2 acc[kPairs][kAcc];
#pragma unroll
            for (int j = 0; j < kPairs; ++j)
#pragma unroll
                for (int r = 0; r < kAcc; ++r) acc[j][r] = 0ull;
            int pr[kPairs];
#pragma unroll
            for (int j = 0; j < kPairs; ++j) {
                const int p = pass * kPassPairs + tid + j * kT;
                pr[j] = p < npairs ? p : 0;
            }

            for (int cb = 0; cb < nc; cb += chunk) {
                const int ncc = min(chunk, nc - cb);
                for (int t0 = 0; t0 < si.T; t0 += TT) {
                    const int tt = min(TT, si.T - t0);
                    // ---- stage the tile, then expand into operand pairs
                    if (!stage_tile<kT, true>(a, si, head, raw, coef, t0, tt, cb, ncc, kref, d2pi, hmax, nmax, phase))
                        break;
                    for (int i = tid; i < tt * ncc; i += kT) {
                        const float4 v0 = raw[2 * i], v1 = raw[2 * i + 1];
                        float4 *d = vexp + 6 * i;
                        if (kG) {
                            // per correlation: a, a + b, b - a (each duplicated)
                            const float re[4] = {v0.x, v0.z, v1.x, v1.z}, im[4] = {v0.y, v0.w, v1.y, v1.w};
                            float e[12];
#pragma unroll
                            for (int k = 0; k < 4; ++k) {
                                e[3 * k] = re[k];
                                e[3 * k + 1] = re[k] + im[k];
                                e[3 * k + 2] = im[k] - re[k];
                            }
#pragma unroll
                            for (int q = 0; q < 6; ++q) d[q] = make_float4(e[2 * q], e[2 * q], e[2 * q + 1], e[2 * q + 1]);
                        } else {
                            d[0] = make_float4(v0.x, v0.x, v0.y, v0.y);
                            d[1] = make_float4(v0.z, v0.z, v0.w, v0.w);
                            d[2] = make_float4(v1.x, v1.x, v1.y, v1.y);
                            d[3] = make_float4(v1.z, v1.z, v1.w, v1.w);
                            d[4] = make_float4(-v0.y, -v0.y, -v0.w, -v0.w);
                            d[5] = make_float4(-v1.y, -v1.y, -v1.w, -v1.w);
                        }
                    }
                    if (tid == 0) {
                        head->fast = (3.1416f + kappa_max * __int_as_float(head->qmax_bits)) <= kFastBound ? 1 : 0;
                        head->qmax_bits = 0; // next tile's atomics come after two more barriers
                    }
                    __syncthreads();
                    const bool fast = head->fast != 0;

                    // ---- compute
                    if constexpr (kRec) {
                        if (fast)
                            grid_tile_recur<kPairs, kUnr, (PIPE & kFtz) != 0, (PIPE & kPipe) != 0>(acc, pr, coef, geo, vexp, kap + cb,
                                                                             chains + cb, tt, ncc);
                        else
                            grid_tile<kPairs, false, PIPE, kAcc, kUnr>(acc, pr, coef, geo, vexp, kap + cb, tt, ncc);
                    } else if (fast)
                        grid_tile<kPairs, true, PIPE, kAcc, kUnr>(acc, pr, coef, geo, vexp, kap + cb, tt, ncc);
                    else
                        grid_tile<kPairs, false, PIPE, kAcc, kUnr>(acc, pr, coef, geo, vexp, kap + cb, tt, ncc);
                }
                if (head->abort) break;
            }
            if (head->abort) break;

            // ---- epilogue: A-terms, taper, store two pixels per pair
            const size_t jones_stride = (size_t)S2 * 2;
            const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
            const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;
            const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;
#pragma unroll
            for (int j = 0; j < kPairs; ++j) {
                const int p = pass * kPassPairs + tid + j * kT;
                if (p >= npairs) continue;
                cf px[2][4];
#pragma unroll
                for (int pol = 0; pol < 4; ++pol) {
                    float r0, r1, i0, i1;
                    if (kG) {
                        // Re = k1 - k2, Im = k1 + k3
                        unpack2(fsub2(acc[j][3 * pol], acc[j][3 * pol + 1]), r0, r1);
                        unpack2(fadd2(acc[j][3 * pol], acc[j][3 * pol + 2]), i0, i1);
                    } else {
                        unpack2(acc[j][2 * pol], r0, r1);
                        unpack2(acc[j][2 * pol + 1], i0, i1);
                    }
                    px[0][pol] = {r0, i0};
                    px[1][pol] = {r1, i1};
                }
                float out[2][8];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int q = 2 * p + h;
                    cf j1[4], j2[4];
                    load_jones(a1 + 2 * q, j1);
                    load_jones(a2 + 2 * q, j2);
                    aterm_gridder(px[h], j1, j2);
                    const float sph = taper ? a.taper[q] : 1.f;
#pragma unroll
                    for (int pol = 0; pol < 4; ++pol) {
                        out[h][2 * pol] = px[h][pol].re * sph;
                        out[h][2 * pol + 1] = px[h][pol].im * sph;
                    }
                }
#pragma unroll
                for (int pol = 0; pol < 4; ++pol) {
                    float4 *dst = reinterpret_cast<float4 *>(a.subgrids + ((size_t)s * 4 + pol) * S2 + 2 * p);
                    *dst = make_float4(out[0][2 * pol], out[0][2 * pol + 1], out[1][2 * pol], out[1][2 * pol + 1]);
                }
            }
        }
        if (head->abort) break;
    }
}

// ---------------------------------------------------------------------------
// Mirror-quad form (shapes 18-22).  The pixels of a subgrid come in quads
// (hx, hy), (-hx, hy), (hx, -hy), (-hx, -hy) (pixel x and S-1-x have opposite
// hx exactly, and all four share n).  The phase of channel c is
//   x_c = a_c hx + b_c hy + g_c n,  a_c = A + kappa_c qu, b_c = B + kappa_c qv,
//   g_c = G + kappa_c qw
// (the same per-timestep coefficients as above, regrouped by pixel factor), so
// with P = e^{i a_c hx}, Q = e^{i b_c hy}, R = e^{i g_c n}, X = P Q, Y = conj(P) Q
// and W = V R the four pixels receive W X, W conj(X), W Y, W conj(Y).  W X and
// W conj(X) share their four real products (Wr Xr, Wi Xi, Wr Xi, Wi Xr): summed
// separately over all visibilities they give both pixels in the epilogue, so a
// quad costs 8 FMA per correlation per visibility (2 per pixel, against 3 for
// the Gauss form), plus W = V R (4 per correlation, shared by the quad) and
// the four products m1 = Pc Qc, m2 = Ps Qs, m3 = Pc Qs, m4 = Ps Qc (4) that
// X and Y are made of: the accumulators sum W times each m, and the epilogue
// forms Wr Xr = sum Wr (m1 - m2) and so on.  Per pixel-visibility: 13.75 FMA
// and 1.5 SFU operations (three sincos per quad), against 14 FMA and 2 SFU
// operations per pixel above, and 8 accumulators per pixel instead of 12.
// Each thread owns GP pairs of quads; the two quads of a pair sit in the two
// halves of the packed FP32x2 registers.  Per (timestep, quad pair) the
// factors' offsets tau = A hx, B hy, G n are reduced to [-pi, pi] once; per
// channel the arguments are tau + kappa_c (qu hx, qv hy, qw n), below the
// unreduced-sincos bound on fast tiles and reduced otherwise.
// ---------------------------------------------------------------------------
// SHP: every quad of the thread has the same x column (NT a multiple of S/2),
// so P is one sincos per thread, shared by all its quads.
// qg: the thread's quad geometry in shared memory, qg[(3 j + c) * NT] for
// quad pair j and c = hx, hy, n (read once per timestep, not held in registers
// across the channel loop).
template <int GP, bool FAST, int UNR, bool SHP, int NT>
__device__ __forceinline__ void quad_tile(f2 (&acc)[GP][4][8], const f2 *qg, const float4 *coef, const float4 *vq,
                                          const f2 *kp, int tt, int ncc) {
    for (int t = 0; t < tt; ++t) {
        const float4 c0 = coef[3 * t], c1 = coef[3 * t + 1], c2 = coef[3 * t + 2];
        const f2 A2 = pack2(c0.x, c0.y), B2 = pack2(c0.z, c0.w), G2 = pack2(c1.x, c1.y);
        const f2 QU = pack2(c1.z, c1.w), QV = pack2(c2.x, c2.y), QW = pack2(c2.z, c2.w);
        f2 tx[GP], ty[GP], tn[GP], qx[GP], qy[GP], qn[GP];
#pragma unroll
        for (int j = 0; j < GP; ++j) {
            const f2 hx = qg[(3 * j) * NT], hy = qg[(3 * j + 1) * NT], nn = qg[(3 * j + 2) * NT];
            tx[j] = reduce_2pi(fmul2(A2, hx));
            ty[j] = reduce_2pi(fmul2(B2, hy));
            tn[j] = reduce_2pi(fmul2(G2, nn));
            qx[j] = fmul2(QU, hx);
            qy[j] = fmul2(QV, hy);
            qn[j] = fmul2(QW, nn);
        }
        const float4 *vt = vq + (size_t)t * ncc * 4;
#pragma unroll UNR
        for (int c = 0; c < ncc; ++c) {
            const f2 kc = kp[c];
            // visibility operands, duplicated into both halves: (vr, vr), (vi, vi) per correlation
            f2 vr[4], vi[4];
            const uint32_t base = smem_addr(vt + 4 * c);
#pragma unroll
            for (int k = 0; k < 4; ++k) lds2(base + 16 * k, vr[k], vi[k]);
            f2 Pc0 = 0ull, Ps0 = 0ull;
            if (SHP) {
                f2 ap = ffma2(kc, qx[0], tx[0]);
                if (!FAST) ap = reduce_2pi(ap);
                float a0, a1, sn, cs;
                unpack2(ap, a0, a1);
                __sincosf(a0, &sn, &cs);
                Pc0 = dup(cs);
                Ps0 = dup(sn);
            }
#pragma unroll
            for (int j = 0; j < GP; ++j) {
                f2 aq = ffma2(kc, qy[j], ty[j]), ar = ffma2(kc, qn[j], tn[j]);
                if (!FAST) {
                    aq = reduce_2pi(aq);
                    ar = reduce_2pi(ar);
                }
                f2 Pc = Pc0, Ps = Ps0, Qc, Qs, Rc, Rs;
                if (!SHP) {
                    f2 ap = ffma2(kc, qx[j], tx[j]);
                    if (!FAST) ap = reduce_2pi(ap);
                    sincos_pair<false>(ap, Pc, Ps);
                }
                sincos_pair<false>(aq, Qc, Qs);
                sincos_pair<false>(ar, Rc, Rs);
                // the products X and Y are made of: Xr = m1 - m2, Yr = m1 + m2,
                // Xi = m3 + m4, Yi = m3 - m4
                const f2 m1 = fmul2(Pc, Qc), m2 = fmul2(Ps, Qs), m3 = fmul2(Pc, Qs), m4 = fmul2(Ps, Qc);
                const f2 nRs = neg2(Rs);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    // W = V R
                    const f2 Wr = ffma2(vr[k], Rc, fmul2(vi[k], nRs));
                    const f2 Wi = ffma2(vr[k], Rs, fmul2(vi[k], Rc));
                    f2 *q = acc[j][k];
                    q[0] = ffma2(Wr, m1, q[0]);
                    q[1] = ffma2(Wr, m2, q[1]);
                    q[2] = ffma2(Wi, m1, q[2]);
                    q[3] = ffma2(Wi, m2, q[3]);
                    q[4] = ffma2(Wr, m3, q[4]);
                    q[5] = ffma2(Wr, m4, q[5]);
                    q[6] = ffma2(Wi, m3, q[6]);
                    q[7] = ffma2(Wi, m4, q[7]);
                }
            }
        }
    }
}

// Kernel of the mirror-quad form: NT threads, GP quad pairs per thread per
// pass, TV visibilities per staged tile, at least MINB CTAs per SM.  Staging,
// coefficients, work distribution and failure handling as gridder_fast_kernel.
template <int NT, int GP, int TV, int MINB, int UNR>
__global__ void __launch_bounds__(NT, MINB) gridder_quad_kernel(KernelArgs a) {
    constexpr int kT = NT, kPassQuads = NT * GP * 2, kTileVis = TV, kMaxChunk = TV;
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = a.S, S2 = S * S, Sh = S / 2, nquads = Sh * Sh;
    // quad g of a pass has x column g mod Sh; with NT a multiple of Sh every quad
    // of a thread (offsets multiples of NT) is in the thread's column
    const bool shared_x = NT % Sh == 0;
    const QuadLayout L = quad_layout(a.C, TV);
    SmemHead *head = reinterpret_cast<SmemHead *>(smem);
    float4 *raw = reinterpret_cast<float4 *>(smem + L.raw);
    float4 *vq = reinterpret_cast<float4 *>(smem + L.vexp);
    float4 *coef = reinterpret_cast<float4 *>(smem + L.coef);
    f2 *kap = reinterpret_cast<f2 *>(smem + L.kappa);
    const int tid = threadIdx.x;

    if (tid == 0) {
        mbar_init(&head->bar, 1);
        mbar_init_fence();
        head->abort = 0;
    }
    __syncthreads();
    uint32_t phase = 0;
    const double d2pi = (double)a.image_size / (double)S / kTwoPi;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            head->next = atomicAdd(a.work_counter, 1);
            head->kmax_bits = 0;
            head->qmax_bits = 0;
        }
        __syncthreads();
        const int idx = head->next;
        if (idx >= a.nr_subgrids || head->abort) break;
        const int s = a.work_list ? a.work_list[idx] : idx;
        const SubgridInfo si = load_subgrid(a, s);
        const int nc = si.c1 - si.c0;
        if (!si.ok) {
            if (tid == 0) flag_status(a.status, kStatusBadPlan);
            for (int i = tid; i < 4 * S2; i += kT) a.subgrids[(size_t)s * 4 * S2 + i] = make_float2(0.f, 0.f);
            continue;
        }
        const int cref = si.c0 + (nc > 0 ? (nc - 1) / 2 : 0);
        const double kref = nc > 0 ? (double)a.wavenumbers[cref] : 0.0;
        float kmax = 0.f;
        for (int c = tid; c < nc; c += kT) {
            const float kv = (float)((double)a.wavenumbers[si.c0 + c] - kref);
            kap[c] = dup(kv);
            kmax = fmaxf(kmax, fabsf(kv));
        }
        if (kmax > 0.f) atomicMax(&head->kmax_bits, __float_as_int(kmax));
        __syncthreads();
        const float kappa_max = __int_as_float(head->kmax_bits);

        const int chunk = nc < kMaxChunk ? nc : kMaxChunk;
        const int TT = nc > 0 ? min(kMaxTT, kTileVis / chunk) : 1;
        const float hmax = 0.5f * (float)(S - 1);
        const float nmax = pixel_geometry(0, S, a.image_size).z;

        for (int pass = 0; pass * kPassQuads < nquads; ++pass) {
            f2 acc[GP][4][8];
#pragma unroll
            for (int j = 0; j < GP; ++j)
#pragma unroll
                for (int k = 0; k < 4; ++k)
#pragma unroll
                    for (int r = 0; r < 8; ++r) acc[j][k][r] = 0ull;
            // the quads of this thread: pair j holds quads g0 (low half) and g1 (high half);
            // each quad is named by its pixel (gx, gy) in the low-x, low-y quadrant
            int qd[GP][2];
            f2 *qg = reinterpret_cast<f2 *>(smem + L.total) + tid;
#pragma unroll
            for (int j = 0; j < GP; ++j) {
                float gxh[2], gyh[2], gnn[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int g = pass * kPassQuads + (2 * j + h) * kT + tid;
                    qd[j][h] = g < nquads ? g : -1;
                    const int gg = g < nquads ? g : 0;
                    const int gy = gg / Sh, gx = gg - gy * Sh;
                    const float3 geo = pixel_geometry(gy * S + gx, S, a.image_size);
                    gxh[h] = geo.x;
                    gyh[h] = geo.y;
                    gnn[h] = geo.z;
                }
                qg[(3 * j) * kT] = pack2(gxh[0], gxh[1]);
                qg[(3 * j + 1) * kT] = pack2(gyh[0], gyh[1]);
                qg[(3 * j + 2) * kT] = pack2(gnn[0], gnn[1]);
            }

            for (int cb = 0; cb < nc; cb += chunk) {
                const int ncc = min(chunk, nc - cb);
                for (int t0 = 0; t0 < si.T; t0 += TT) {
                    const int tt = min(TT, si.T - t0);
                    if (!stage_tile<kT, false>(a, si, head, raw, coef, t0, tt, cb, ncc, kref, d2pi, hmax, nmax, phase))
                        break;
                    // expand: per visibility and correlation (re, re, im, im)
                    for (int i = tid; i < tt * ncc; i += kT) {
                        const float4 v0 = raw[2 * i], v1 = raw[2 * i + 1];
                        float4 *d = vq + 4 * i;
                        d[0] = make_float4(v0.x, v0.x, v0.y, v0.y);
                        d[1] = make_float4(v0.z, v0.z, v0.w, v0.w);
                        d[2] = make_float4(v1.x, v1.x, v1.y, v1.y);
                        d[3] = make_float4(v1.z, v1.z, v1.w, v1.w);
                    }
                    if (tid == 0) {
                        // each factor's argument stays within pi + max|kappa| max|q h|
                        head->fast = (3.1416f + kappa_max * __int_as_float(head->qmax_bits)) <= kFastBound ? 1 : 0;
                        head->qmax_bits = 0;
                    }
                    __syncthreads();
                    if (shared_x) {
                        if (head->fast)
                            quad_tile<GP, true, UNR, true, kT>(acc, qg, coef, vq, kap + cb, tt, ncc);
                        else
                            quad_tile<GP, false, UNR, true, kT>(acc, qg, coef, vq, kap + cb, tt, ncc);
                    } else if (head->fast) {
                        quad_tile<GP, true, UNR, false, kT>(acc, qg, coef, vq, kap + cb, tt, ncc);
                    } else {
                        quad_tile<GP, false, UNR, false, kT>(acc, qg, coef, vq, kap + cb, tt, ncc);
                    }
                }
                if (head->abort) break;
            }
            if (head->abort) break;

            // ---- epilogue: the four pixels of each quad, A-terms, taper
            const size_t jones_stride = (size_t)S2 * 2;
            const float4 *a1 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st1) * jones_stride;
            const float4 *a2 = a.aterms + ((size_t)si.aterm * a.nr_stations + si.st2) * jones_stride;
            const bool taper = (a.flags & IDG_FLAG_NO_TAPER) == 0;
#pragma unroll
            for (int j = 0; j < GP; ++j) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (qd[j][h] < 0) continue;
                    const int gy = qd[j][h] / Sh, gx = qd[j][h] - gy * Sh;
                    // pixels: 0 = (gx, gy) -> W X ; 1 = (S-1-gx, S-1-gy) -> W conj(X)
                    //         2 = (S-1-gx, gy) -> W Y ; 3 = (gx, S-1-gy) -> W conj(Y)
                    const int qx[4] = {gx, S - 1 - gx, S - 1 - gx, gx};
                    const int qy[4] = {gy, S - 1 - gy, gy, S - 1 - gy};
                    cf px[4][4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        float m[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            float lo, hi;
                            unpack2(acc[j][k][i], lo, hi);
                            m[i] = h ? hi : lo;
                        }
                        // sums of Wr m1, Wr m2, Wi m1, Wi m2, Wr m3, Wr m4, Wi m3, Wi m4 ->
                        // Wr Xr, Wi Xi, Wr Xi, Wi Xr, Wr Yr, Wi Yi, Wr Yi, Wi Yr
                        const float r[8] = {m[0] - m[1], m[6] + m[7], m[4] + m[5], m[2] - m[3],
                                            m[0] + m[1], m[6] - m[7], m[4] - m[5], m[2] + m[3]};
                        px[0][k] = {r[0] - r[1], r[2] + r[3]};
                        px[1][k] = {r[0] + r[1], r[3] - r[2]};
                        px[2][k] = {r[4] - r[5], r[6] + r[7]};
                        px[3][k] = {r[4] + r[5], r[7] - r[6]};
                    }
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int q = qy[e] * S + qx[e];
                        cf j1[4], j2[4];
                        load_jones(a1 + 2 * q, j1);
                        load_jones(a2 + 2 * q, j2);
                        aterm_gridder(px[e], j1, j2);
                        const float sph = taper ? a.taper[q] : 1.f;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            a.subgrids[((size_t)s * 4 + k) * S2 + q] = make_float2(px[e][k].re * sph, px[e][k].im * sph);
                    }
                }
            }
        }
        if (head->abort) break;
    }
}

// Launch shapes the autotuner chooses from (index = batched-gridder shape id):
//   0: 128 threads x 4 pairs, 256-visibility tiles, 3 CTAs/SM (12 warps), plain channel loop
//   1: 128 x 4, 2 CTAs/SM (8 warps), software-pipelined channel loop, registers uncapped
//   2: 128 x 2, 128-visibility tiles, 4 CTAs/SM (16 warps), pipelined
//   3: 256 x 2, 256-visibility tiles, 2 CTAs/SM (16 warps), pipelined
//   4: 128 x 2, 128-visibility tiles, 4 CTAs/SM (16 warps), plain channel loop
//   5: shape 0 with the subnormal-flushing SFU sine/cosine
//   6: shape 1 with the subnormal-flushing SFU sine/cosine
//   7: 128 x 4, 2 CTAs/SM, Gauss MACs, channel loop unrolled by two
//   8: 128 x 4, 2 CTAs/SM, Gauss MACs, pipelined and unrolled by two
//   9: 256 x 2, 2 CTAs/SM (16 warps), Gauss MACs, unrolled by two
//  10: 128 x 4, 3 CTAs/SM, Gauss MACs
//  11: 96 x 3 (288 pairs per pass: whole passes for S = 24 and 48), Gauss, pipelined, unrolled by two
//  12: 128 x 3 (384 pairs per pass: whole passes for S = 48), Gauss, pipelined, unrolled by two
//  13: shape 8 with the channel loop unrolled by four
//  14: shape 7 with the channel loop unrolled by four
//  15: 128 x 4, 2 CTAs/SM, Gauss MACs, channel recurrence (chains <= 16), unrolled by four
//  16: shape 15 with each channel's next phasor computed ahead of its MACs
//  17: 128 x 3 (whole passes for S = 48), 2 CTAs/SM, Gauss MACs, channel recurrence, unrolled by four
//  18: mirror quads, 128 threads x 2 quads, 3 CTAs/SM (12 warps), channel loop unrolled by four
//  19: mirror quads, 128 threads x 2 quads, 2 CTAs/SM (8 warps), registers uncapped
//  20: mirror quads, 64 threads x 4 quads, 4 CTAs/SM (8 warps), unrolled by two (whole passes for S = 32)
//  21: mirror quads, 128 threads x 4 quads, 2 CTAs/SM (8 warps), unrolled by two (whole passes for S = 64)
//  22: shape 20 with the channel loop unrolled by four
//  23: shape 22 with 384-visibility tiles (fewer stages per subgrid)
//  24: shape 22 with 512-visibility tiles
// load_only: only make sure the kernel is loaded into the current context
// (under lazy module loading a kernel is otherwise loaded, which takes device
// memory, at its first launch).
template <int NT, int PAIRS, int TV, int MINB, int PIPE>
cudaError_t launch_shape(const KernelArgs &a, cudaStream_t stream, bool load_only) {
    auto kern = gridder_fast_kernel<NT, PAIRS, TV, MINB, PIPE>;
    if (load_only) {
        cudaFuncAttributes fa;
        return cudaFuncGetAttributes(&fa, kern);
    }
    const size_t smem = layout(a.S, a.C, TV).total;
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

template <int NT, int GP, int TV, int MINB, int UNR>
cudaError_t launch_quad(const KernelArgs &a, cudaStream_t stream, bool load_only) {
    auto kern = gridder_quad_kernel<NT, GP, TV, MINB, UNR>;
    if (load_only) {
        cudaFuncAttributes fa;
        return cudaFuncGetAttributes(&fa, kern);
    }
    if (a.S % 2 != 0) return cudaErrorInvalidValue;
    const size_t smem = quad_layout(a.C, TV).total + (size_t)NT * GP * 3 * sizeof(f2); // + quad geometry
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

int gridder_fast_shapes() { return 25; }

namespace {
cudaError_t dispatch_gridder_fast(const KernelArgs &a, cudaStream_t stream, int shape, bool load_only) {
    switch (shape) {
    case 1: return launch_shape<128, 4, 256, 2, 1>(a, stream, load_only);
    case 2: return launch_shape<128, 2, 128, 4, 1>(a, stream, load_only);
    case 3: return launch_shape<256, 2, 256, 2, 1>(a, stream, load_only);
    case 4: return launch_shape<128, 2, 128, 4, 0>(a, stream, load_only);
    case 5: return launch_shape<128, 4, 256, 3, 2>(a, stream, load_only);
    case 6: return launch_shape<128, 4, 256, 2, 3>(a, stream, load_only);
    case 7: return launch_shape<128, 4, 256, 2, kGauss | kUnroll2>(a, stream, load_only);
    case 8: return launch_shape<128, 4, 256, 2, kGauss | kPipe | kUnroll2>(a, stream, load_only);
    case 9: return launch_shape<256, 2, 256, 2, kGauss | kUnroll2>(a, stream, load_only);
    case 10: return launch_shape<128, 4, 256, 3, kGauss>(a, stream, load_only);
    case 11: return launch_shape<96, 3, 256, 3, kGauss | kPipe | kUnroll2>(a, stream, load_only);
    case 12: return launch_shape<128, 3, 256, 2, kGauss | kPipe | kUnroll2>(a, stream, load_only);
    case 13: return launch_shape<128, 4, 256, 2, kGauss | kPipe | kUnroll4>(a, stream, load_only);
    case 14: return launch_shape<128, 4, 256, 2, kGauss | kUnroll4>(a, stream, load_only);
    case 15: return launch_shape<128, 4, 256, 2, kGauss | kRecur | kUnroll4>(a, stream, load_only);
    case 16: return launch_shape<128, 4, 256, 2, kGauss | kRecur | kPipe | kUnroll4>(a, stream, load_only);
    case 17: return launch_shape<128, 3, 256, 2, kGauss | kRecur | kUnroll4>(a, stream, load_only);
    case 18: return launch_quad<128, 1, 256, 3, 4>(a, stream, load_only);
    case 19: return launch_quad<128, 1, 256, 2, 4>(a, stream, load_only);
    case 20: return launch_quad<64, 2, 256, 4, 2>(a, stream, load_only);
    case 21: return launch_quad<128, 2, 256, 2, 2>(a, stream, load_only);
    case 22: return launch_quad<64, 2, 256, 4, 4>(a, stream, load_only);
    case 23: return launch_quad<64, 2, 384, 4, 4>(a, stream, load_only);
    case 24: return launch_quad<64, 2, 512, 4, 4>(a, stream, load_only);
    default: return launch_shape<128, 4, 256, 3, 0>(a, stream, load_only);
    }
}
} // namespace

cudaError_t launch_gridder_fast(const KernelArgs &a, cudaStream_t stream, int shape) {
    return dispatch_gridder_fast(a, stream, shape, false);
}

cudaError_t load_gridder_fast() {
    const KernelArgs a{};
    for (int shape = 0; shape < gridder_fast_shapes(); ++shape)
        if (cudaError_t e = dispatch_gridder_fast(a, nullptr, shape, true)) return e;
    return cudaSuccess;
}

} // namespace idg
