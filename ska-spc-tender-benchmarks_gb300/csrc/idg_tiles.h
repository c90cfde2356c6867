// idg_tiles.h -- the adder with a fixed summation order: host binning of a
// plan's subgrids into grid tiles, and the device view its two passes read
// (idg_tiles.cu).
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/idg_gb300.h"

namespace idg {

struct TileItem {
    int tile;  // plane * tiles_per_plane + ty * ntx + tx
    int begin; // entries [begin, end) of the tile's list
    int end;
    int slot;  // -1: add into the grid; else the partial tile written
};

struct TileMulti {
    int tile;
    int first_slot;
    int nslots;
    int reserved;
};

// The bins of one plan on the host.
struct TileBinsHost {
    int S = 0, G = 0, W = 1, ntx = 0;
    std::vector<int> entries;    // per tile, its subgrids in ascending order
    std::vector<TileItem> items; // pass-1 work items, longest first
    std::vector<TileMulti> multi;
    int nslots = 0;              // partial tiles of pass 1
    size_t partial_bytes() const;
};

// What the kernels read: device copies of the bins and the plan's metadata,
// and room for the partial tiles.
struct TileBinsDev {
    const idg_metadata *md = nullptr;
    const int *entries = nullptr;
    const TileItem *items = nullptr;
    const TileMulti *multi = nullptr;
    float2 *partials = nullptr;
    int S = 0, G = 0, ntx = 0, nitems = 0, nmulti = 0;
};

// Bins `nr_subgrids` HOST plan entries; IDG_OK or an error code (with text).
int bin_tiles(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata, TileBinsHost *out);
// grid += subgrids in the bins' fixed order (two kernels on `stream`).
cudaError_t launch_binned_adder(const TileBinsDev &b, const float2 *subgrids, float2 *grid, cudaStream_t stream);
// One cudaMalloc holding `metadata` and the bins; `view` points into it.
int upload_tile_bins(const TileBinsHost &h, int64_t nr_subgrids, const idg_metadata *metadata, void **mem,
                     TileBinsDev *view);

} // namespace idg
