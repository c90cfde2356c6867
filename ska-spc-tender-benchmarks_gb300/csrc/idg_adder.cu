// idg_adder.cu -- adder (subgrids -> grid) and splitter (grid -> subgrids).
//
// Adder   : grid[z][pol][y0+j][x0+i] += F[s][pol][j][i]   for cells inside the G x G grid
// Splitter: F[s][pol][j][i] = grid[z][pol][y0+j][x0+i]     (0 for cells outside)
// (x0, y0, z) are the plan entry's coordinate.  w-stacking with negative w:
// the grid holds w-planes z = 0 .. W-1 (offsets (z + 1/2) w_step >= 0); an
// entry with -W <= z < 0 uses the Hermitian symmetry V(-u,-v,-w) = V(u,v,w)^H
// and goes to plane -z-1 at the mirrored cell (G - gy, G - gx), conjugated,
// with the cross-hand correlations swapped (xy <-> yx):
//   adder    grid[-z-1][pol'][G-gy][G-gx] += conj(F[s][pol][j][i])
//   splitter F[s][pol][j][i] = conj(grid[-z-1][pol'][G-gy][G-gx])
// (gy = y0 + j, gx = x0 + i, pol' = the swapped index; mirrored cells outside
// the grid are skipped / read as 0).  Both are bandwidth kernels:
// one CTA per subgrid, consecutive threads on consecutive cells of a row, so
// subgrid and grid accesses coalesce.  Subgrid footprints of one plan overlap
// (consecutive time slices of a baseline land on nearly the same cells), so
// the adder accumulates with vector reductions into L2 (red.global.add on
// float4 = two cells when x0 is even, float2 otherwise); the splitter is a
// plain gather.
#include "idg_device.cuh"
#include "idg_internal.h"

namespace idg {

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) adder_kernel(const idg_metadata *md, int S, int G, int W,
                                                         const float2 *subgrids, float2 *grid) {
    const int s = blockIdx.x;
    const idg_metadata m = md[s];
    if (m.z < -W || m.z >= W) return;
    const int64_t S2 = (int64_t)S * S;
    const float2 *src = subgrids + (int64_t)s * 4 * S2;
    if (m.z < 0) { // mirrored into plane -z-1
        float2 *mp = grid + (int64_t)(-m.z - 1) * 4 * G * G;
        for (int e = threadIdx.x; e < 4 * S * S; e += kThreads) {
            const int pol = e / (S * S), r = e - pol * S * S, j = r / S, i = r - j * S;
            const int gy = G - (m.y + j), gx = G - (m.x + i);
            if (gy < 0 || gy >= G || gx < 0 || gx >= G) continue;
            const int pm = (pol == 1 || pol == 2) ? 3 - pol : pol;
            const float2 v = src[pol * S2 + r];
            atomicAdd(mp + ((int64_t)pm * G + gy) * G + gx, make_float2(v.x, -v.y));
        }
        return;
    }
    float2 *plane0 = grid + (int64_t)m.z * 4 * G * G;
    if ((m.x & 1) == 0 && (S & 1) == 0 && (G & 1) == 0) {
        // two cells per thread, 16-byte aligned on both sides (even x, S and G)
        const int half = S / 2;
        for (int e = threadIdx.x; e < 4 * S * half; e += kThreads) {
            const int pol = e / (S * half), r = e - pol * S * half, j = r / half, i2 = (r - j * half) * 2;
            const int gy = m.y + j, gx = m.x + i2;
            if (gy < 0 || gy >= G || gx < 0 || gx + 1 >= G) {
                // partially or fully outside: fall back to per-cell
                for (int d = 0; d < 2; ++d) {
                    const int gxd = gx + d;
                    if (gy >= 0 && gy < G && gxd >= 0 && gxd < G)
                        atomicAdd(plane0 + ((int64_t)pol * G + gy) * G + gxd, src[pol * S2 + (int64_t)j * S + i2 + d]);
                }
                continue;
            }
            const float4 v = reinterpret_cast<const float4 *>(src + pol * S2 + (int64_t)j * S)[i2 / 2];
            atomicAdd(reinterpret_cast<float4 *>(plane0 + ((int64_t)pol * G + gy) * G + gx), v);
        }
    } else {
        for (int e = threadIdx.x; e < 4 * S * S; e += kThreads) {
            const int pol = e / (S * S), r = e - pol * S * S, j = r / S, i = r - j * S;
            const int gy = m.y + j, gx = m.x + i;
            if (gy < 0 || gy >= G || gx < 0 || gx >= G) continue;
            atomicAdd(plane0 + ((int64_t)pol * G + gy) * G + gx, src[pol * S2 + r]);
        }
    }
}

__global__ void __launch_bounds__(kThreads) splitter_kernel(const idg_metadata *md, int S, int G, int W,
                                                            const float2 *grid, float2 *subgrids) {
    const int s = blockIdx.x;
    const idg_metadata m = md[s];
    const int64_t S2 = (int64_t)S * S;
    float2 *dst = subgrids + (int64_t)s * 4 * S2;
    const bool plane_ok = m.z >= -W && m.z < W;
    const bool mirror = m.z < 0;
    const float2 *plane0 = grid + (int64_t)(plane_ok ? (mirror ? -m.z - 1 : m.z) : 0) * 4 * G * G;
    for (int e = threadIdx.x; e < 4 * S * S; e += kThreads) {
        const int pol = e / (S * S), r = e - pol * S * S, j = r / S, i = r - j * S;
        const int gy = mirror ? G - (m.y + j) : m.y + j, gx = mirror ? G - (m.x + i) : m.x + i;
        const int pg = (mirror && (pol == 1 || pol == 2)) ? 3 - pol : pol;
        float2 v = make_float2(0.f, 0.f);
        if (plane_ok && gy >= 0 && gy < G && gx >= 0 && gx < G) v = plane0[((int64_t)pg * G + gy) * G + gx];
        if (mirror) v.y = -v.y;
        dst[e] = v;
    }
}

} // namespace

cudaError_t launch_adder(const idg_metadata *md, int64_t nr_subgrids, int S, int G, int W, const float2 *subgrids,
                         float2 *grid, cudaStream_t stream) {
    if (nr_subgrids == 0) return cudaSuccess;
    adder_kernel<<<(unsigned)nr_subgrids, kThreads, 0, stream>>>(md, S, G, W, subgrids, grid);
    return cudaGetLastError();
}

cudaError_t launch_splitter(const idg_metadata *md, int64_t nr_subgrids, int S, int G, int W, const float2 *grid,
                            float2 *subgrids, cudaStream_t stream) {
    if (nr_subgrids == 0) return cudaSuccess;
    splitter_kernel<<<(unsigned)nr_subgrids, kThreads, 0, stream>>>(md, S, G, W, grid, subgrids);
    return cudaGetLastError();
}

} // namespace idg
