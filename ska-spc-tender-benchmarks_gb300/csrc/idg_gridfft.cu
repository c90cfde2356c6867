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
// e^{-2 pi i m / G} computed in FP64 on the host, read through the read-only
// cache (one table serves every row of the pass).  All passes are HBM-bound:
// 16 bytes per complex cell per pass (read + write).
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"

namespace idg {

namespace {

constexpr int kRowThreads = 256;
constexpr int kTile = 32;

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
// twiddles element r by e^{DIR 2 pi i r k / (L R)} (table e^{-2 pi i m / G},
// conjugated for DIR = +1), transforms the R values in registers and writes
// them to q L R + k + r L.
template <int DIR, int G, int L, int R>
__device__ __forceinline__ void stockham_pass(const float2 *src, float2 *dst, const float2 *tw_g) {
    constexpr int n = G / (L * R);
    for (int b = threadIdx.x; b < G / R; b += kRowThreads) {
        const int k = b % L, q = b / L;
        float2 x[R];
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = src[pad16(b + r * (G / R))];
        if (L > 1 && k > 0) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                const float2 w = __ldg(tw_g + (r * k) * n);
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

// One FFT over the CTA's row (length G = 2^LOGG, row stride G).  DIR = -1
// uses e^{-2 pi i ...}, DIR = +1 its conjugate.  Element i of the row is
// multiplied by (-1)^i before and after the transform (the centre shifts of
// this dimension), and by corr[i] (when given) after it for DIR = -1 or before
// it for DIR = +1.  The row is staged in padded shared memory with all of a
// thread's 16-byte loads issued before any is used, then transformed by
// radix-16 Stockham passes in registers (three for G = 4096).
template <int DIR, int LOGG>
__global__ void __launch_bounds__(kRowThreads) grid_row_fft_kernel(float2 *data, const float2 *tw_g,
                                                                   const float *corr) {
    constexpr int G = 1 << LOGG, kVec = G / 2;  // float4 per row
    constexpr int kPer = (kVec + kRowThreads - 1) / kRowThreads;
    extern __shared__ float2 sm[];
    float2 *A = sm, *B = sm + (G + G / 16);
    const int row = blockIdx.x;
    float2 *p = data + (int64_t)row * G;
    float4 v[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int i2 = threadIdx.x + k * kRowThreads;
        if (i2 < kVec) v[k] = reinterpret_cast<const float4 *>(p)[i2];
    }
    // pre-multiply for the image -> uv direction
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int i2 = threadIdx.x + k * kRowThreads;
        if (i2 >= kVec) continue;
        float fa = 1.f, fb = -1.f; // (-1)^i for i = 2 i2, 2 i2 + 1
        if (DIR > 0 && corr) {
            fa *= corr[2 * i2];
            fb *= corr[2 * i2 + 1];
        }
        A[pad16(2 * i2)] = make_float2(v[k].x * fa, v[k].y * fa);
        A[pad16(2 * i2 + 1)] = make_float2(v[k].z * fb, v[k].w * fb);
    }
    __syncthreads();
    float2 *src = A, *dst = B;
    stockham_passes<DIR, G, 1>(src, dst, tw_g);
    // post-multiply for the uv -> image direction, store
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int i2 = threadIdx.x + k * kRowThreads;
        if (i2 >= kVec) continue;
        const float2 a = src[pad16(2 * i2)], b = src[pad16(2 * i2 + 1)];
        float fa = 1.f, fb = -1.f;
        if (DIR < 0 && corr) {
            fa *= corr[2 * i2];
            fb *= corr[2 * i2 + 1];
        }
        reinterpret_cast<float4 *>(p)[i2] = make_float4(a.x * fa, a.y * fa, b.x * fb, b.y * fb);
    }
}

template <int DIR, int LOGG>
cudaError_t row_pass(float2 *grid, int64_t rows, const float2 *tw, const float *corr, cudaStream_t st) {
    const size_t smem = 2 * sizeof(float2) * (((size_t)1 << LOGG) + ((size_t)1 << LOGG) / 16);
    cudaError_t e = cudaFuncSetAttribute(grid_row_fft_kernel<DIR, LOGG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    grid_row_fft_kernel<DIR, LOGG><<<(unsigned)rows, kRowThreads, smem, st>>>(grid, tw, corr);
    return cudaGetLastError();
}

template <int DIR>
cudaError_t row_pass_g(int logG, float2 *grid, int64_t rows, const float2 *tw, const float *corr, cudaStream_t st) {
    switch (logG) {
    case 6: return row_pass<DIR, 6>(grid, rows, tw, corr, st);
    case 7: return row_pass<DIR, 7>(grid, rows, tw, corr, st);
    case 8: return row_pass<DIR, 8>(grid, rows, tw, corr, st);
    case 9: return row_pass<DIR, 9>(grid, rows, tw, corr, st);
    case 10: return row_pass<DIR, 10>(grid, rows, tw, corr, st);
    case 11: return row_pass<DIR, 11>(grid, rows, tw, corr, st);
    case 12: return row_pass<DIR, 12>(grid, rows, tw, corr, st);
    case 13: return row_pass<DIR, 13>(grid, rows, tw, corr, st);
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

cudaError_t launch_grid_fft(float2 *grid, int G, int planes, int direction, const float *corr, cudaStream_t st) {
    if (!grid_fft_size_supported(G)) return cudaErrorInvalidValue;
    const float2 *tw = nullptr;
    cudaError_t e = twiddles(G, &tw);
    if (e != cudaSuccess) return e;
    int logG = 0;
    while ((1 << logG) < G) ++logG;
    const int64_t rows = (int64_t)planes * G;
    auto rowpass = [&]() -> cudaError_t {
        return direction < 0 ? row_pass_g<-1>(logG, grid, rows, tw, corr, st)
                             : row_pass_g<1>(logG, grid, rows, tw, corr, st);
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
