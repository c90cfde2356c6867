// idg_tiles.cu -- the adder with a fixed summation order ("tile bins").
//
// The adder's job is grid[z][pol][y0+j][x0+i] += F[s][pol][j][i] over all
// subgrids s (with the Hermitian mirror for -W <= z < 0; see idg_adder.cu).
// Footprints overlap heavily -- consecutive time slices of a baseline land on
// nearly the same cells, and short baselines crowd the centre of the grid -- so
// idg_adder() accumulates with floating-point atomics, whose order (and so the
// last bits of the result) changes from run to run.  Here the order is fixed:
//
//  * On the host, once per plan, the subgrids are binned into tiles of 32 x 32
//    cells of their target plane (a counting sort in subgrid order, so each
//    tile's list is ascending).  Each list is cut into chunks of at most
//    kChunk subgrids.
//  * Pass 1, one CTA per chunk: the chunk's plan entries are staged in shared
//    memory; every thread owns two cells of one column of the tile (all four
//    correlations) and adds the chunk's subgrids into registers, in list
//    order.  A tile with one chunk is then added into the
//    grid with plain loads and stores -- no other CTA touches it; a tile with
//    several chunks writes each chunk's sum to a partial tile.
//  * Pass 2, one CTA per tile with several chunks: grid += partial 0, then
//    partial 1, ... in chunk order.
// No atomics; the result depends on the plan only.  Loads of a subgrid row
// coalesce across the warp (consecutive lanes, consecutive cells).  Cells that
// fall outside the grid and entries outside [-W, W) are skipped, as in
// idg_adder().
#include <algorithm>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"
#include "idg_tiles.h"

namespace idg {
namespace {

constexpr int kTile = 32;       // tile edge in cells (one warp lane per column)
constexpr int kWarps = 16;      // rows of a tile shared out over 16 warps, 2 rows each
constexpr int kRowsPerThread = kTile / kWarps;
constexpr int kChunk = 128;     // subgrids per pass-1 work item

__device__ __forceinline__ int swap_pol(int p) { return (p == 1 || p == 2) ? 3 - p : p; }

// The chunk's plan entries (x, y, z, subgrid) are staged in shared memory
// first; the entry loop then issues predicated loads (cells outside an entry's
// footprint load nothing and add zero) takes two entries per step, so that
// both entries' loads are in flight before either is added.  The adds stay in
// list order.
__global__ void __launch_bounds__(kTile * kWarps, 2)
    tile_add_kernel(const TileItem *items, const int *entries, const idg_metadata *md, int S, int G, int ntx,
                    const float2 *subgrids, float2 *grid, float2 *partials) {
    __shared__ int4 smd[kChunk];
    const TileItem it = items[blockIdx.x];
    const int n = it.end - it.begin;
    for (int e = threadIdx.x; e < n; e += kTile * kWarps) {
        const int s = entries[it.begin + e];
        const idg_metadata m = md[s];
        smd[e] = make_int4(m.x, m.y, m.z, s);
    }
    const int per_plane = ntx * ntx;
    const int plane = it.tile / per_plane, r = it.tile - plane * per_plane, ty = r / ntx, tx = r - ty * ntx;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gx = tx * kTile + lane;
    const int64_t S2 = (int64_t)S * S;
    float2 acc[kRowsPerThread][4];
#pragma unroll
    for (int k = 0; k < kRowsPerThread; ++k)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[k][p] = make_float2(0.f, 0.f);
    __syncthreads();

    // two entries per step: both entries' loads are issued before either is added
    for (int e = 0; e < n; e += 2) {
        float2 v[2][kRowsPerThread][4];
        bool mir[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int4 m = smd[e + h < n ? e + h : e];
            const bool live = e + h < n;
            mir[h] = m.z < 0;
            const int i = mir[h] ? G - gx - m.x : gx - m.x;
            const bool xin = live && (unsigned)i < (unsigned)S && gx < G;
            const float2 *src = subgrids + (int64_t)m.w * 4 * S2 + (xin ? i : 0);
#pragma unroll
            for (int k = 0; k < kRowsPerThread; ++k) {
                const int gy = ty * kTile + warp + kWarps * k;
                const int j = mir[h] ? G - gy - m.y : gy - m.y;
                const bool in = xin && (unsigned)j < (unsigned)S && gy < G;
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    // grid correlation p takes subgrid correlation p, or its swap when mirrored
                    const int q = mir[h] ? swap_pol(p) : p;
                    v[h][k][p] = in ? __ldg(src + q * S2 + (int64_t)j * S) : make_float2(0.f, 0.f);
                }
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int k = 0; k < kRowsPerThread; ++k)
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    acc[k][p].x += v[h][k][p].x;
                    acc[k][p].y += mir[h] ? -v[h][k][p].y : v[h][k][p].y; // mirrored: conjugated
                }
    }

    if (gx >= G) return;
#pragma unroll
    for (int k = 0; k < kRowsPerThread; ++k) {
        const int row = warp + kWarps * k, gy = ty * kTile + row;
        if (gy >= G) continue;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            if (it.slot < 0) {
                float2 *c = grid + (((int64_t)plane * 4 + p) * G + gy) * G + gx;
                const float2 g = *c;
                *c = make_float2(g.x + acc[k][p].x, g.y + acc[k][p].y);
            } else {
                partials[(((int64_t)it.slot * 4 + p) * kTile + row) * kTile + lane] = acc[k][p];
            }
        }
    }
}

__global__ void __launch_bounds__(kTile * kWarps)
    tile_combine_kernel(const TileMulti *multi, int G, int ntx, const float2 *partials, float2 *grid) {
    const TileMulti t = multi[blockIdx.x];
    const int per_plane = ntx * ntx;
    const int plane = t.tile / per_plane, r = t.tile - plane * per_plane, ty = r / ntx, tx = r - ty * ntx;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gx = tx * kTile + lane;
    if (gx >= G) return;
#pragma unroll
    for (int k = 0; k < kRowsPerThread; ++k) {
        const int row = warp + kWarps * k, gy = ty * kTile + row;
        if (gy >= G) continue;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            float2 *c = grid + (((int64_t)plane * 4 + p) * G + gy) * G + gx;
            float2 g = *c;
            for (int q = 0; q < t.nslots; ++q) {
                const float2 v = partials[(((int64_t)(t.first_slot + q) * 4 + p) * kTile + row) * kTile + lane];
                g.x += v.x;
                g.y += v.y;
            }
            *c = g;
        }
    }
}

// The footprint of entry m in grid cells of its target plane, [lo, hi) per
// axis after clipping to the grid; false when empty or outside [-W, W).
bool footprint(const idg_metadata &m, int S, int G, int W, int *plane, int *xlo, int *xhi, int *ylo, int *yhi) {
    if (m.z < -W || m.z >= W) return false;
    const bool mirror = m.z < 0;
    *plane = mirror ? -m.z - 1 : m.z;
    // direct: cells x .. x+S-1; mirrored: cells G-x-S+1 .. G-x
    const int64_t x0 = mirror ? (int64_t)G - m.x - S + 1 : m.x, y0 = mirror ? (int64_t)G - m.y - S + 1 : m.y;
    *xlo = (int)std::max<int64_t>(x0, 0);
    *xhi = (int)std::min<int64_t>(x0 + S, G);
    *ylo = (int)std::max<int64_t>(y0, 0);
    *yhi = (int)std::min<int64_t>(y0 + S, G);
    return *xlo < *xhi && *ylo < *yhi;
}

} // namespace

size_t TileBinsHost::partial_bytes() const { return (size_t)nslots * 4 * kTile * kTile * sizeof(float2); }

int bin_tiles(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata, TileBinsHost *out) {
    const int S = params->subgrid_size, G = params->grid_size, W = params->nr_w_planes > 0 ? params->nr_w_planes : 1;
    const int ntx = (G + kTile - 1) / kTile;
    const int64_t per_plane = (int64_t)ntx * ntx, ntiles = per_plane * W;
    if (ntiles > INT32_MAX) return fail(IDG_ERR_UNSUPPORTED, "grid of %d planes of %d^2 cells has too many tiles", W, G);
    // counting sort of (tile, subgrid) pairs by tile, in subgrid order
    std::vector<int64_t> count(ntiles, 0);
    auto each_tile = [&](int64_t s, auto &&fn) {
        int pl, xlo, xhi, ylo, yhi;
        if (!footprint(metadata[s], S, G, W, &pl, &xlo, &xhi, &ylo, &yhi)) return;
        for (int ty = ylo / kTile; ty <= (yhi - 1) / kTile; ++ty)
            for (int tx = xlo / kTile; tx <= (xhi - 1) / kTile; ++tx) fn(pl * per_plane + (int64_t)ty * ntx + tx);
    };
    for (int64_t s = 0; s < nr_subgrids; ++s) each_tile(s, [&](int64_t t) { ++count[t]; });
    std::vector<int64_t> offset(ntiles + 1, 0);
    for (int64_t t = 0; t < ntiles; ++t) offset[t + 1] = offset[t] + count[t];
    const int64_t nentries = offset[ntiles];
    if (nentries > INT32_MAX)
        return fail(IDG_ERR_UNSUPPORTED, "%lld (tile, subgrid) pairs: too many for one bin set", (long long)nentries);
    TileBinsHost &b = *out;
    b = TileBinsHost{};
    b.S = S;
    b.G = G;
    b.W = W;
    b.ntx = ntx;
    b.entries.assign(std::max<int64_t>(nentries, 1), 0);
    std::vector<int64_t> fill(offset.begin(), offset.end() - 1);
    for (int64_t s = 0; s < nr_subgrids; ++s) each_tile(s, [&](int64_t t) { b.entries[fill[t]++] = (int)s; });
    for (int64_t t = 0; t < ntiles; ++t) {
        const int64_t n = count[t];
        if (n == 0) continue;
        const int64_t nch = (n + kChunk - 1) / kChunk;
        if (nch == 1) {
            b.items.push_back({(int)t, (int)offset[t], (int)(offset[t] + n), -1});
            continue;
        }
        b.multi.push_back({(int)t, b.nslots, (int)nch, 0});
        for (int64_t c = 0; c < nch; ++c) {
            const int64_t lo = offset[t] + c * kChunk, hi = std::min(offset[t] + n, lo + kChunk);
            b.items.push_back({(int)t, (int)lo, (int)hi, b.nslots++});
        }
    }
    // longest work items first, so that the short ones fill in at the end
    std::stable_sort(b.items.begin(), b.items.end(),
                     [](const TileItem &x, const TileItem &y) { return x.end - x.begin > y.end - y.begin; });
    return IDG_OK;
}

cudaError_t launch_binned_adder(const TileBinsDev &b, const float2 *subgrids, float2 *grid, cudaStream_t stream) {
    if (b.nitems > 0) {
        tile_add_kernel<<<(unsigned)b.nitems, kTile * kWarps, 0, stream>>>(b.items, b.entries, b.md, b.S, b.G, b.ntx,
                                                                         subgrids, grid, b.partials);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (b.nmulti > 0) {
        tile_combine_kernel<<<(unsigned)b.nmulti, kTile * kWarps, 0, stream>>>(b.multi, b.G, b.ntx, b.partials, grid);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

} // namespace idg

// Bins on the device: the public handle owns the device copies.
struct idg_tile_bins {
    int device = 0;
    int64_t nr_subgrids = 0;
    int64_t info[4] = {0, 0, 0, 0};
    void *mem = nullptr; // metadata, entries, items, multi, partial tiles (one allocation)
    idg::TileBinsDev dev;
};

namespace idg {

// One device allocation holding the plan's metadata and its bins (256-byte
// aligned parts); `mem` receives it, `view` points into it.
int upload_tile_bins(const TileBinsHost &h, int64_t nr_subgrids, const idg_metadata *metadata, void **mem,
                     TileBinsDev *view) {
    auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t b_md = up(sizeof(idg_metadata) * std::max<int64_t>(nr_subgrids, 1)),
                 b_en = up(sizeof(int) * h.entries.size()),
                 b_it = up(sizeof(TileItem) * std::max<size_t>(h.items.size(), 1)),
                 b_mu = up(sizeof(TileMulti) * std::max<size_t>(h.multi.size(), 1)), b_pa = up(h.partial_bytes());
    char *base = nullptr;
    IDG_CUDA(cudaMalloc(reinterpret_cast<void **>(&base), b_md + b_en + b_it + b_mu + b_pa));
    TileBinsDev &v = *view;
    v.md = reinterpret_cast<const idg_metadata *>(base);
    v.entries = reinterpret_cast<const int *>(base + b_md);
    v.items = reinterpret_cast<const TileItem *>(base + b_md + b_en);
    v.multi = reinterpret_cast<const TileMulti *>(base + b_md + b_en + b_it);
    v.partials = h.nslots ? reinterpret_cast<float2 *>(base + b_md + b_en + b_it + b_mu) : nullptr;
    v.S = h.S;
    v.G = h.G;
    v.ntx = h.ntx;
    v.nitems = (int)h.items.size();
    v.nmulti = (int)h.multi.size();
    cudaError_t e = cudaSuccess;
    if (nr_subgrids > 0)
        e = cudaMemcpy(base, metadata, sizeof(idg_metadata) * nr_subgrids, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + b_md, h.entries.data(), sizeof(int) * h.entries.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !h.items.empty())
        e = cudaMemcpy(base + b_md + b_en, h.items.data(), sizeof(TileItem) * h.items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !h.multi.empty())
        e = cudaMemcpy(base + b_md + b_en + b_it, h.multi.data(), sizeof(TileMulti) * h.multi.size(),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(base);
        return cuda_fail(e, "tile bins upload");
    }
    *mem = base;
    return IDG_OK;
}

} // namespace idg

extern "C" {

IDG_API int idg_tile_bins_create(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                                 idg_tile_bins **bins) {
    using namespace idg;
    if (!bins) return fail(IDG_ERR_INVALID_ARGUMENT, "bins output is NULL");
    *bins = nullptr;
    if (!params) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    if (params->subgrid_size < 1 || params->grid_size < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "bad sizes");
    if (nr_subgrids < 0 || nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids");
    if (nr_subgrids > 0 && !metadata) return fail(IDG_ERR_INVALID_ARGUMENT, "metadata is NULL");
    TileBinsHost h;
    if (int rc = bin_tiles(params, nr_subgrids, metadata, &h)) return rc;
    auto *b = new idg_tile_bins;
    cudaGetDevice(&b->device);
    b->nr_subgrids = nr_subgrids;
    b->info[0] = (int64_t)h.items.size();
    b->info[1] = (int64_t)h.multi.size();
    b->info[2] = h.nslots;
    b->info[3] = (int64_t)h.partial_bytes();
    if (int rc = upload_tile_bins(h, nr_subgrids, metadata, &b->mem, &b->dev)) {
        delete b;
        return rc;
    }
    *bins = b;
    return IDG_OK;
}

IDG_API int idg_tile_bins_destroy(idg_tile_bins *bins) {
    if (!bins) return IDG_OK;
    if (bins->mem) cudaFree(bins->mem);
    delete bins;
    return IDG_OK;
}

IDG_API int idg_tile_bins_info(const idg_tile_bins *bins, int64_t *sizes) {
    using namespace idg;
    if (!bins || !sizes) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int i = 0; i < 4; ++i) sizes[i] = bins->info[i];
    return IDG_OK;
}

IDG_API int idg_adder_binned(const idg_tile_bins *bins, const void *subgrids, void *grid, void *stream) {
    using namespace idg;
    if (!bins) return fail(IDG_ERR_INVALID_ARGUMENT, "bins is NULL");
    if (bins->nr_subgrids == 0) return IDG_OK;
    if (!subgrids || !grid) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    int dev = 0;
    IDG_CUDA(cudaGetDevice(&dev));
    if (dev != bins->device)
        return fail(IDG_ERR_INVALID_ARGUMENT, "bins belong to device %d, current is %d", bins->device, dev);
    cudaError_t e = launch_binned_adder(bins->dev, reinterpret_cast<const float2 *>(subgrids),
                                        reinterpret_cast<float2 *>(grid), reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "binned adder launch");
    return IDG_OK;
}

} // extern "C"
