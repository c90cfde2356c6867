// idg_gridfft.cu -- 2-D FFT of the uv-grid (the imaging step after the adder).
//
// For every plane (w-plane, polarisation) of grid[W][4][G][G], G = 2^k:
//   direction -1 (uv -> image):
//     out[y][x] = c[y] c[x] sum_{v,u} grid[v][u] exp(-2 pi i ((u-G/2)(x-G/2) + (v-G/2)(y-G/2)) / G)
//   direction +1 (image -> uv): the adjoint,
//     out[v][u] = sum_{y,x} c[y] c[x] grid[y][x] exp(+2 pi i ((u-G/2)(x-G/2) + (v-G/2)(y-G/2)) / G)
// with c the optional separable grid correction (length G; 1 when NULL).  The
// centre cell G/2 is the origin of both domains.  For G divisible by 4 the
// shifts factorise into (-1)^(u+v) before and (-1)^(x+y) after an unshifted
// DFT, so each 1-D pass is: multiply by (-1)^index (and c), unshifted FFT,
// multiply by (-1)^index (and c).
//
// Passes per plane: row FFTs, tiled transpose, row FFTs, tiled transpose.  A
// row FFT runs in one CTA: the row is staged in shared memory and transformed
// by radix-16 Stockham passes in registers (the last one of radix 2, 4 or 8
// when log2 G is not a multiple of 4), ping-ponging between two shared
// buffers; twiddles come from a table of
// e^{-2 pi i m / G} computed in FP64 on the host, held per CTA as two
// 64-entry-scale shared tables whose product gives any entry.  All passes are
// HBM-bound:
// 16 bytes per complex cell per pass (read + write).
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"
#include "idg_ptx.cuh"

namespace idg {

namespace {

constexpr int kRowThreads = 256;
constexpr int kTile = 32;
constexpr uint64_t kWaitNs = 2000000000ull; // a staged row not complete after 2 s is declared lost

__device__ __forceinline__ float2 cm(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// Shared-memory layout of a staged row: one float2 of padding after every 16,
// so that a thread's 16 consecutive outputs of the first pass, and the
// column-strided inputs of every pass, fall in distinct banks.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// cos / sin of 2 pi m / 16 (compile-time constants once m is).
__host__ __device__ constexpr float kcos16(int m) {
    constexpr float t[16] = {1.f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f,
                             0.f, -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f,
                             -1.f, -0.92387953251128674f, -0.70710678118654752f, -0.38268343236508977f,
                             0.f, 0.38268343236508977f, 0.70710678118654752f, 0.92387953251128674f};
    return t[m & 15];
}
__host__ __device__ constexpr float ksin16(int m) { return kcos16(m - 4); }

__host__ __device__ constexpr int brev(int i, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}

// y[j] = sum_r x[r] e^{SIGN 2 pi i r j / M} in registers, M in {2, 4, 8, 16}:
// bit-reversal permutation, then radix-2 decimation-in-time stages with
// compile-time twiddles.
template <int M, int SIGN, int I = 0>
__device__ __forceinline__ void brev_perm(float2 (&x)[M]) {
    if constexpr (I < M) {
        constexpr int J = brev(I, M == 2 ? 1 : M == 4 ? 2 : M == 8 ? 3 : 4);
        if constexpr (J > I) {
            const float2 t = x[I];
            x[I] = x[J];
            x[J] = t;
        }
        brev_perm<M, SIGN, I + 1>(x);
    }
}
template <int M, int SIGN, int LEN = 2>
__device__ __forceinline__ void dit_stages(float2 (&x)[M]) {
    if constexpr (LEN <= M) {
#pragma unroll
        for (int i0 = 0; i0 < M; i0 += LEN) {
#pragma unroll
            for (int j = 0; j < LEN / 2; ++j) {
                const float2 u = x[i0 + j];
                float2 v = x[i0 + j + LEN / 2];
                if (j > 0) v = cm(v, make_float2(kcos16(j * (16 / LEN)), SIGN * ksin16(j * (16 / LEN))));
                x[i0 + j] = make_float2(u.x + v.x, u.y + v.y);
                x[i0 + j + LEN / 2] = make_float2(u.x - v.x, u.y - v.y);
            }
        }
        dit_stages<M, SIGN, 2 * LEN>(x);
    }
}

// One Stockham pass of radix R over sub-length L (the product of the radices
// before it): butterfly b = (q, k), k = b mod L, reads elements b + r G/R,
// twiddles element r by e^{DIR 2 pi i r k / (L R)} (e^{-2 pi i m / G} from the
// two shared tables at tw_g, conjugated for DIR = +1), transforms the R
// values in registers and writes them to q L R + k + r L.
// FIRST: src is the row as copied from global memory (unpadded), and each
// element i is multiplied on the way in by (-1)^i (and by corr[i] for the
// image -> uv direction).
// Twiddle e^{-2 pi i m / G}, m < G, from two shared tables built once per
// CTA: lo[j] = e^{-2 pi i j / G} (j < 64) and hi[j] = e^{-2 pi i 64 j / G}.
__device__ __forceinline__ float2 twiddle(const float2 *lo, const float2 *hi, int m) {
    return cm(lo[m & 63], hi[m >> 6]);
}

template <int DIR, int G, int L, int R, bool FIRST = false>
__device__ __forceinline__ void stockham_pass(const float2 *src, float2 *dst, const float2 *tw_g,
                                              const float *corr = nullptr) {
    constexpr int n = G / (L * R);
    for (int b = threadIdx.x; b < G / R; b += kRowThreads) {
        const int k = b % L, q = b / L;
        float2 x[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (FIRST) {
                const int i = b + r * (G / R);
                float f = (i & 1) ? -1.f : 1.f;
                if (DIR > 0 && corr) f *= __ldg(corr + i);
                const float2 e = src[i];
                x[r] = make_float2(e.x * f, e.y * f);
            } else {
                x[r] = src[pad16(b + r * (G / R))];
            }
        }
        if (L > 1 && k > 0) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                const float2 w = twiddle(tw_g, tw_g + 64, (r * k) * n);
                x[r] = cm(x[r], DIR < 0 ? w : conjf2(w));
            }
        }
        brev_perm<R, DIR>(x);
        dit_stages<R, DIR>(x);
#pragma unroll
        for (int r = 0; r < R; ++r) dst[pad16(q * L * R + k + r * L)] = x[r];
    }
}

// The passes of a length-G transform: radix 16 while at least 16 points of
// the length are left, then one pass of radix 2, 4 or 8.  Swaps src / dst
// after every pass, so the result is in src at the end.
template <int DIR, int G, int L>
__device__ __forceinline__ void stockham_passes(float2 *&src, float2 *&dst, const float2 *tw_g) {
    if constexpr (L < G) {
        constexpr int rem = G / L, R = rem >= 16 ? 16 : rem;
        stockham_pass<DIR, G, L, R>(src, dst, tw_g);
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
        stockham_passes<DIR, G, L * R>(src, dst, tw_g);
    }
}

// Row FFTs (length G = 2^LOGG, row stride G) by persistent CTAs.  DIR = -1
// uses e^{-2 pi i ...}, DIR = +1 its conjugate.  Element i of a row is
// multiplied by (-1)^i before and after the transform (the centre shifts of
// this dimension), and by corr[i] (when given) after it for DIR = -1 or before
// it for DIR = +1.  Each CTA takes rows blockIdx.x, + gridDim.x, ...: a row
// arrives in a staging buffer by one bulk async copy (completion counted on an
// mbarrier, waits bounded by kWaitNs), the first radix-16 pass reads it from
// there (pre-multiplication folded in) into a padded buffer, and the next
// row's copy is issued as soon as the staging buffer is free, so it overlaps
// the remaining passes and the store of the current row.  A copy that does not
// arrive in time sets the timeout bit of `status` and the CTA stops (`lost`
// extra expected bytes on the first copy make that happen in tests).
template <int DIR, int LOGG>
__global__ void __launch_bounds__(kRowThreads) grid_row_fft_kernel(float2 *data, int64_t rows, const float2 *tw_g,
                                                                   const float *corr, unsigned *status,
                                                                   uint32_t lost) {
    constexpr int G = 1 << LOGG, kVec = G / 2;  // float4 per row
    constexpr int kPer = (kVec + kRowThreads - 1) / kRowThreads;
    constexpr int R1 = G >= 16 ? 16 : G;
    constexpr uint32_t kRowBytes = (uint32_t)G * 8u;
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float2 *C = reinterpret_cast<float2 *>(smem + 16); // staged row (bulk-copy target)
    float2 *A = C + G, *B = A + (G + G / 16);          // padded ping-pong buffers
    __shared__ float2 tws[64 + G / 64];                 // twiddle tables (see twiddle())
    __shared__ int abort_flag;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
        abort_flag = 0;
    }
    for (int j = tid; j < 64 + G / 64; j += kRowThreads) tws[j] = tw_g[j < 64 ? j : 64 * (j - 64)];
    __syncthreads();
    uint32_t phase = 0;
    int64_t row = blockIdx.x;
    if (tid == 0 && row < rows) {
        mbar_arrive_expect_tx(bar, kRowBytes + lost); // lost > 0 only under IDG_FLAG_TEST_LOST_COPY
        bulk_g2s(C, data + row * G, kRowBytes, bar);
    }
    for (; row < rows; row += gridDim.x) {
        if (!mbar_wait_bounded(bar, phase, kWaitNs)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) {
            if (tid == 0) {
                flag_status(status, kStatusTimeout);
                mbar_wait_bounded(bar, phase, kWaitNs); // the copy in flight, once more
            }
            break;
        }
        phase ^= 1u;
        stockham_pass<DIR, G, 1, R1, true>(C, B, tws, corr);
        __syncthreads(); // C read by every thread: free for the next row
        if (tid == 0 && row + gridDim.x < rows) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar, kRowBytes);
            bulk_g2s(C, data + (row + gridDim.x) * G, kRowBytes, bar);
        }
        float2 *src = B, *dst = A;
        stockham_passes<DIR, G, R1>(src, dst, tws);
        // post-multiply for the uv -> image direction, store
        float2 *p = data + row * G;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int i2 = tid + k * kRowThreads;
            if (i2 >= kVec) continue;
            const float2 a = src[pad16(2 * i2)], b = src[pad16(2 * i2 + 1)];
            float fa = 1.f, fb = -1.f;
            if (DIR < 0 && corr) {
                fa *= corr[2 * i2];
                fb *= corr[2 * i2 + 1];
            }
            reinterpret_cast<float4 *>(p)[i2] = make_float4(a.x * fa, a.y * fa, b.x * fb, b.y * fb);
        }
        __syncthreads(); // the output buffer is read before the next row's first pass writes B
    }
}

template <int DIR, int LOGG>
cudaError_t row_pass(float2 *grid, int64_t rows, const float2 *tw, const float *corr, unsigned *status,
                     uint32_t lost, cudaStream_t st) {
    constexpr size_t G = (size_t)1 << LOGG;
    const size_t smem = 16 + sizeof(float2) * (G + 2 * (G + G / 16));
    auto kern = grid_row_fft_kernel<DIR, LOGG>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRowThreads, smem)) != cudaSuccess) return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    if (blocks > rows) blocks = rows;
    kern<<<(unsigned)blocks, kRowThreads, smem, st>>>(grid, rows, tw, corr, status, lost);
    return cudaGetLastError();
}

template <int DIR>
cudaError_t row_pass_g(int logG, float2 *grid, int64_t rows, const float2 *tw, const float *corr, unsigned *status,
                       uint32_t lost, cudaStream_t st) {
    switch (logG) {
    case 6: return row_pass<DIR, 6>(grid, rows, tw, corr, status, lost, st);
    case 7: return row_pass<DIR, 7>(grid, rows, tw, corr, status, lost, st);
    case 8: return row_pass<DIR, 8>(grid, rows, tw, corr, status, lost, st);
    case 9: return row_pass<DIR, 9>(grid, rows, tw, corr, status, lost, st);
    case 10: return row_pass<DIR, 10>(grid, rows, tw, corr, status, lost, st);
    case 11: return row_pass<DIR, 11>(grid, rows, tw, corr, status, lost, st);
    case 12: return row_pass<DIR, 12>(grid, rows, tw, corr, status, lost, st);
    case 13: return row_pass<DIR, 13>(grid, rows, tw, corr, status, lost, st);
    default: return cudaErrorInvalidValue;
    }
}

// In-place transpose of planes of G x G: CTA (bx, by) with bx >= by swaps tile
// (by, bx) with tile (bx, by) (the diagonal tiles transpose in place).
__global__ void __launch_bounds__(kTile * 8) grid_transpose_kernel(float2 *data, int G) {
    __shared__ float2 ta[kTile][kTile + 1], tb[kTile][kTile + 1];
    const int bx = blockIdx.x, by = blockIdx.y;
    if (bx < by) return;
    float2 *plane = data + (int64_t)blockIdx.z * G * G;
    const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile; // 32 x 8
    for (int j = ty; j < kTile; j += 8) {
        ta[j][tx] = plane[(int64_t)(by * kTile + j) * G + bx * kTile + tx];
        if (bx != by) tb[j][tx] = plane[(int64_t)(bx * kTile + j) * G + by * kTile + tx];
    }
    __syncthreads();
    for (int j = ty; j < kTile; j += 8) {
        plane[(int64_t)(bx * kTile + j) * G + by * kTile + tx] = ta[tx][j];
        if (bx != by) plane[(int64_t)(by * kTile + j) * G + bx * kTile + tx] = tb[tx][j];
    }
}

std::mutex g_tw_mutex;
std::map<std::pair<int, int>, float2 *> g_tw; // (device, G) -> e^{-2 pi i m / G}, m < G

cudaError_t twiddles(int G, const float2 **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_tw_mutex);
    auto it = g_tw.find({dev, G});
    if (it != g_tw.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    std::vector<float2> h(G);
    for (int m = 0; m < G; ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)G;
        h[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    float2 *d = nullptr;
    e = cudaMalloc(&d, sizeof(float2) * G);
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(d, h.data(), sizeof(float2) * G, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return e;
    }
    g_tw[{dev, G}] = d;
    *out = d;
    return cudaSuccess;
}

} // namespace

bool grid_fft_size_supported(int G) { return G >= 64 && G <= 8192 && (G & (G - 1)) == 0; }

cudaError_t launch_grid_fft(float2 *grid, int G, int planes, int direction, const float *corr, unsigned *status,
                            bool test_lost_copy, cudaStream_t st) {
    const uint32_t lost = test_lost_copy ? 16u : 0u;
    if (!grid_fft_size_supported(G)) return cudaErrorInvalidValue;
    const float2 *tw = nullptr;
    cudaError_t e = twiddles(G, &tw);
    if (e != cudaSuccess) return e;
    int logG = 0;
    while ((1 << logG) < G) ++logG;
    const int64_t rows = (int64_t)planes * G;
    auto rowpass = [&]() -> cudaError_t {
        return direction < 0 ? row_pass_g<-1>(logG, grid, rows, tw, corr, status, lost, st)
                             : row_pass_g<1>(logG, grid, rows, tw, corr, status, lost, st);
    };
    const dim3 tgrid(G / kTile, G / kTile, planes);
    // rows (x), transpose, rows (y), transpose back
    if ((e = rowpass()) != cudaSuccess) return e;
    grid_transpose_kernel<<<tgrid, kTile * 8, 0, st>>>(grid, G);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = rowpass()) != cudaSuccess) return e;
    grid_transpose_kernel<<<tgrid, kTile * 8, 0, st>>>(grid, G);
    return cudaGetLastError();
}

} // namespace idg
