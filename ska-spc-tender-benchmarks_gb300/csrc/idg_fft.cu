// idg_fft.cu -- batched subgrid FFT, fused with the taper.
//
// direction +1 (image -> uv, after gridding):
//   F[j][i] = sum_{y,x} t(y,x) P[y][x] exp(+2 pi i((j-S/2)(y-S/2+1/2) + (i-S/2)(x-S/2+1/2))/S)
// direction -1 (uv -> image, before degridding): the adjoint, taper applied last.
// For even S this factorises (up to a constant that squares to 1 in 2-D) into
//   forward : pre-multiply by (-1)^(x+y) t(y,x), unnormalised DFT with e^{+2 pi i jy/S},
//             post-multiply by c_j c_i,  c_j = (-1)^j e^{+i pi (j-S/2)/S}
//   backward: pre-multiply by conj(c_j c_i), DFT with e^{-2 pi i jy/S},
//             post-multiply by (-1)^(x+y) t(y,x)
// The pixel centres sit half a cell off the DFT lattice (l = (x+1/2-S/2)/S * image_size),
// which is where the e^{i pi j/S} factors come from.
//
// Kernel: a CTA transforms PLANES (subgrid, polarisation) planes.  One
// thread per row loads its row straight into registers (16-byte loads; the
// rows of a CTA stay in L1 while a warp's loads walk them), pre-multiplies
// it and runs a register-resident radix-2 (x radix-3 for S = 24, 48) FFT; the
// rows pass through padded shared memory once, as a transpose; one thread per
// column then transforms its column and stores it post-multiplied, a warp
// writing whole rows.
//
// Split + backward FFT (SPLIT): the degridding step's splitter and backward
// FFT in one pass.  The load stage reads each plane's footprint on the uv-grid
// (the splitter's rule: w-plane z, or the Hermitian mirror -z-1 with
// coordinates G - (x, y), polarisations 1 and 2 swapped and the value
// conjugated, for z < 0; zeros outside the grid or the planes) instead of a
// subgrid, so the subgrid is written once, already in the image domain.
#include "idg_device.cuh"
#include "idg_internal.h"

namespace idg {

namespace {

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }
// Bit reversal of i in `bits` <= 6 bits, as one straight-line expression so
// that it folds to a constant inside fully unrolled loops (a loop here left the
// register arrays indexed at run time, i.e. in local memory).
__host__ __device__ constexpr int bitrev(int i, int bits) {
    return ((((i >> 0) & 1) << 5) | (((i >> 1) & 1) << 4) | (((i >> 2) & 1) << 3) | (((i >> 3) & 1) << 2) |
            (((i >> 4) & 1) << 1) | ((i >> 5) & 1)) >> (6 - bits);
}

// Compile-time bit-reversal permutation of x[0..M) (template recursion: every
// index is a constant, so x stays in registers).
template <int M, int I = 0>
__device__ __forceinline__ void bitrev_permute(cf *x) {
    if constexpr (I < M) {
        constexpr int J = bitrev(I, ilog2(M));
        if constexpr (J > I) {
            const cf t = x[I];
            x[I] = x[J];
            x[J] = t;
        }
        bitrev_permute<M, I + 1>(x);
    }
}

// Radix-2 butterflies of stage LEN (and, recursively, the later stages).
template <int M, int N, int SIGN, int LEN>
__device__ __forceinline__ void fft_stages(cf *x, const float2 *tw) {
#pragma unroll
    for (int i0 = 0; i0 < M; i0 += LEN) {
#pragma unroll
        for (int j = 0; j < LEN / 2; ++j) {
            const float2 w2 = tw[j * (N / LEN)];
            const cf w = {w2.x, SIGN > 0 ? w2.y : -w2.y};
            const cf u = x[i0 + j];
            const cf v = (j == 0) ? x[i0 + j + LEN / 2] : cmul(x[i0 + j + LEN / 2], w);
            x[i0 + j] = cadd(u, v);
            x[i0 + j + LEN / 2] = {u.re - v.re, u.im - v.im};
        }
    }
    if constexpr (LEN < M) fft_stages<M, N, SIGN, 2 * LEN>(x, tw);
}

// In-register radix-2 DIT FFT of M = 2^k points x[0..M) whose twiddles come
// from tw[m] = e^{+2 pi i m / N} (M divides N).  SIGN = +1 or -1.
template <int M, int N, int SIGN>
__device__ __forceinline__ void fft_pow2(cf *x, const float2 *tw) {
    static_assert(M <= 64, "bitrev handles up to 6 bits");
    bitrev_permute<M>(x);
    if constexpr (M > 1) fft_stages<M, N, SIGN, 2>(x, tw);
}

// Length-N FFT with N = 2^k or 3 * 2^k, in registers.
template <int N, int SIGN>
__device__ __forceinline__ void fft_1d(cf *x, const float2 *tw) {
    if constexpr ((N & (N - 1)) == 0) {
        fft_pow2<N, N, SIGN>(x, tw);
    } else {
        static_assert(N % 3 == 0 && ((N / 3) & (N / 3 - 1)) == 0, "N must be 2^k or 3*2^k");
        constexpr int M = N / 3;
        cf y0[M], y1[M], y2[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            y0[m] = x[3 * m];
            y1[m] = x[3 * m + 1];
            y2[m] = x[3 * m + 2];
        }
        fft_pow2<M, N, SIGN>(y0, tw);
        fft_pow2<M, N, SIGN>(y1, tw);
        fft_pow2<M, N, SIGN>(y2, tw);
        // omega = e^{SIGN 2 pi i / 3}
        const float wr = -0.5f, wi = SIGN * 0.86602540378443864676f;
#pragma unroll
        for (int k = 0; k < M; ++k) {
            const float2 t1 = tw[k], t2 = tw[2 * k];
            const cf w1 = {t1.x, SIGN > 0 ? t1.y : -t1.y}, w2 = {t2.x, SIGN > 0 ? t2.y : -t2.y};
            const cf a0 = y0[k], a1 = cmul(y1[k], w1), a2 = cmul(y2[k], w2);
            const cf s = cadd(a1, a2);
            const cf d = {a1.re - a2.re, a1.im - a2.im};
            x[k] = cadd(a0, s);
            // a0 + omega a1 + omega^2 a2 = a0 - s/2 + i*wi*d ; the third output uses -i*wi*d
            const cf base = {a0.re + wr * s.re, a0.im + wr * s.im};
            x[k + M] = {base.re - wi * d.im, base.im + wi * d.re};
            x[k + 2 * M] = {base.re + wi * d.im, base.im - wi * d.re};
        }
    }
}

template <int S>
struct FftShape {
    static constexpr int planes = S >= 64 ? 1 : 128 / S; // <= 48 KiB of static shared memory
    static constexpr int threads = planes * S;
    static constexpr int pitch = S + 1; // float2 per padded row
};

// Where a plane of the split + FFT kernel comes from on the uv-grid.
struct PlaneSrc {
    int64_t base;  // offset of the plane's polarisation in the grid, -1: all zeros
    int x0, y0;    // grid coordinates of pixel (0, 0); mirrored planes step backwards
    int mirror;
};

struct SplitArgs {
    const idg_metadata *md;
    const float2 *grid;
    int G, W;
};

template <int S, int DIR, bool SPLIT>
__global__ void __launch_bounds__(FftShape<S>::threads) subgrid_fft_kernel(float2 *data, int64_t nr_planes,
                                                                          const float *taper, SplitArgs sa) {
    static_assert(!SPLIT || DIR < 0, "the split pass runs before the backward transform");
    static_assert(S % 2 == 0, "rows are read as pairs of pixels");
    using Sh = FftShape<S>;
    __shared__ float2 tw[S];      // e^{+2 pi i m / S}
    __shared__ float2 post[S];    // c_j = (-1)^j e^{+i pi (j - S/2)/S}
    __shared__ float2 buf[Sh::planes][S][Sh::pitch];
    __shared__ PlaneSrc src_of[SPLIT ? Sh::planes : 1];

    const int tid = threadIdx.x;
    if (tid < S) {
        // single-precision sincospi: a unit in the last place, far inside the
        // transform's tolerance, and no FP64 work in every CTA
        float s, c;
        sincospif(2.0f * (float)tid / (float)S, &s, &c);
        tw[tid] = make_float2(c, s);
        sincospif(((float)tid - 0.5f * (float)S) / (float)S, &s, &c);
        const float sg = (tid & 1) ? -1.f : 1.f;
        post[tid] = make_float2(sg * c, sg * s);
    }
    const int64_t plane0 = (int64_t)blockIdx.x * Sh::planes;
    const int nplanes = (int)min((int64_t)Sh::planes, nr_planes - plane0);
    if (SPLIT && tid < nplanes) {
        const int64_t p = plane0 + tid;
        const idg_metadata m = sa.md[p >> 2];
        const int pol = (int)(p & 3);
        const bool ok = m.z >= -sa.W && m.z < sa.W, mirror = m.z < 0;
        const int pg = (mirror && (pol == 1 || pol == 2)) ? 3 - pol : pol;
        const int64_t w = ok ? (mirror ? -m.z - 1 : m.z) : 0;
        PlaneSrc ps;
        ps.base = ok ? (w * 4 + pg) * (int64_t)sa.G * sa.G : -1;
        ps.x0 = mirror ? sa.G - m.x : m.x;
        ps.y0 = mirror ? sa.G - m.y : m.y;
        ps.mirror = mirror;
        src_of[tid] = ps;
    }
    __syncthreads();

    const int pl = tid / S, r = tid - (tid / S) * S;
    cf x[S];
    if (!SPLIT) {
        // Contiguous planes: coalesced 16-byte loads, eight in flight per
        // thread, pre-multiplied into padded shared memory; thread (pl, r)
        // then takes row r of plane pl from there.
        constexpr int kBatch = 8;
        const int total2 = nplanes * S * S / 2;  // float4 elements of this CTA's planes
        const float4 *src = reinterpret_cast<const float4 *>(data + plane0 * S * S);
        for (int base = 0; base < total2; base += kBatch * Sh::threads) {
            float4 v[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const int e2 = base + tid + k * Sh::threads;
                v[k] = e2 < total2 ? src[e2] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const int e2 = base + tid + k * Sh::threads;
                if (e2 >= total2) continue;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int e = 2 * e2 + h;
                    const int p2 = e / (S * S), q = e - p2 * S * S, y = q / S, xx = q - y * S;
                    float2 w = h ? make_float2(v[k].z, v[k].w) : make_float2(v[k].x, v[k].y);
                    if (DIR > 0) {
                        const float f = (((xx + y) & 1) ? -1.f : 1.f) * (taper ? __ldg(taper + q) : 1.f);
                        w = make_float2(w.x * f, w.y * f);
                    } else {
                        const float2 cy = post[y], cx = post[xx];
                        const cf c = cconj(cmul({cy.x, cy.y}, {cx.x, cx.y}));
                        const cf rr = cmul({w.x, w.y}, c);
                        w = make_float2(rr.re, rr.im);
                    }
                    buf[p2][y][xx] = w;
                }
            }
        }
        __syncthreads();
        if (pl < nplanes) {
#pragma unroll
            for (int i = 0; i < S; ++i) x[i] = {buf[pl][r][i].x, buf[pl][r][i].y};
        }
    } else if (pl < nplanes) {
        // The split pass gathers grid rows: thread (pl, r) reads row r of its
        // plane's footprint straight into registers and pre-multiplies it.
        const PlaneSrc ps = src_of[pl];
        const int step = ps.mirror ? -1 : 1;
        const int gy = ps.y0 + step * r;
        const bool row_ok = ps.base >= 0 && gy >= 0 && gy < sa.G;
        const float2 *grow = sa.grid + (row_ok ? ps.base + (int64_t)gy * sa.G : 0);
        // all of the row's loads first (independent, in flight together),
        // then the pre-multiplication
#pragma unroll
        for (int i = 0; i < S; ++i) {
            const int gx = ps.x0 + step * i;
            float2 v = make_float2(0.f, 0.f);
            if (row_ok && gx >= 0 && gx < sa.G) v = __ldg(grow + gx);
            x[i] = {v.x, ps.mirror ? -v.y : v.y};
        }
#pragma unroll
        for (int i = 0; i < S; ++i) {
            const float2 cy = post[r], cx = post[i];
            const cf c = cconj(cmul({cy.x, cy.y}, {cx.x, cx.y}));
            x[i] = cmul(x[i], c);
        }
    }
    if (pl < nplanes) {
        fft_1d<S, DIR>(x, tw);
#pragma unroll
        for (int i = 0; i < S; ++i) buf[pl][r][i] = make_float2(x[i].re, x[i].im);
    }
    __syncthreads();
    if (pl < nplanes) {
#pragma unroll
        for (int i = 0; i < S; ++i) x[i] = {buf[pl][i][r].x, buf[pl][i][r].y};
        fft_1d<S, DIR>(x, tw);
        float2 *dst = data + (plane0 + pl) * S * S;
#pragma unroll
        for (int i = 0; i < S; ++i) {
            // element (y = i, x = r)
            float2 v = make_float2(x[i].re, x[i].im);
            if (DIR > 0) {
                const float2 cy = post[i], cx = post[r];
                const cf r2 = cmul(cmul({v.x, v.y}, {cy.x, cy.y}), {cx.x, cx.y});
                v = make_float2(r2.re, r2.im);
            } else {
                const float f = (((r + i) & 1) ? -1.f : 1.f) * (taper ? __ldg(taper + i * S + r) : 1.f);
                v = make_float2(v.x * f, v.y * f);
            }
            dst[i * S + r] = v;
        }
    }
}

template <int S>
cudaError_t launch_fft_s(float2 *data, int64_t nr_planes, int direction, const float *taper, cudaStream_t stream) {
    using Sh = FftShape<S>;
    const int64_t blocks = (nr_planes + Sh::planes - 1) / Sh::planes;
    if (blocks == 0) return cudaSuccess;
    const SplitArgs none{nullptr, nullptr, 0, 0};
    if (direction > 0)
        subgrid_fft_kernel<S, 1, false><<<(unsigned)blocks, Sh::threads, 0, stream>>>(data, nr_planes, taper, none);
    else
        subgrid_fft_kernel<S, -1, false><<<(unsigned)blocks, Sh::threads, 0, stream>>>(data, nr_planes, taper, none);
    return cudaGetLastError();
}

template <int S>
cudaError_t launch_split_fft_s(const idg_metadata *md, int64_t nr_planes, int G, int W, const float2 *grid,
                               float2 *subgrids, const float *taper, cudaStream_t stream) {
    using Sh = FftShape<S>;
    const int64_t blocks = (nr_planes + Sh::planes - 1) / Sh::planes;
    if (blocks == 0) return cudaSuccess;
    const SplitArgs sa{md, grid, G, W};
    subgrid_fft_kernel<S, -1, true><<<(unsigned)blocks, Sh::threads, 0, stream>>>(subgrids, nr_planes, taper, sa);
    return cudaGetLastError();
}

} // namespace

bool fft_size_supported(int S) { return S == 8 || S == 16 || S == 24 || S == 32 || S == 48 || S == 64; }

cudaError_t launch_subgrid_fft(float2 *data, int64_t nr_subgrids, int S, int direction, const float *taper,
                               cudaStream_t stream) {
    const int64_t planes = nr_subgrids * 4;
    switch (S) {
    case 8: return launch_fft_s<8>(data, planes, direction, taper, stream);
    case 16: return launch_fft_s<16>(data, planes, direction, taper, stream);
    case 24: return launch_fft_s<24>(data, planes, direction, taper, stream);
    case 32: return launch_fft_s<32>(data, planes, direction, taper, stream);
    case 48: return launch_fft_s<48>(data, planes, direction, taper, stream);
    case 64: return launch_fft_s<64>(data, planes, direction, taper, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_split_fft(const idg_metadata *md, int64_t nr_subgrids, int S, int G, int W, const float2 *grid,
                             float2 *subgrids, const float *taper, cudaStream_t stream) {
    const int64_t planes = nr_subgrids * 4;
    switch (S) {
    case 8: return launch_split_fft_s<8>(md, planes, G, W, grid, subgrids, taper, stream);
    case 16: return launch_split_fft_s<16>(md, planes, G, W, grid, subgrids, taper, stream);
    case 24: return launch_split_fft_s<24>(md, planes, G, W, grid, subgrids, taper, stream);
    case 32: return launch_split_fft_s<32>(md, planes, G, W, grid, subgrids, taper, stream);
    case 48: return launch_split_fft_s<48>(md, planes, G, W, grid, subgrids, taper, stream);
    case 64: return launch_split_fft_s<64>(md, planes, G, W, grid, subgrids, taper, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace idg
