// idg_pipeline.cu -- the gridding and degridding steps, and the host-buffer
// imaging cycles with copy/compute overlap.
//
// Gridding step   : gridder (taper off) -> subgrid FFT +1 (taper fused) -> adder
// Degridding step : splitter -> subgrid FFT -1 (taper fused) -> degridder (taper off)
// The taper moves from the gridder epilogue / degridder prologue into the
// FFT's pre/post multiplication, where it costs nothing extra.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"

using namespace idg;

namespace {

int check_step_args(const idg_params *params, int64_t nr_subgrids, const void *subgrids, const void *grid) {
    if (int rc = check_params(params, true)) return rc;
    if (nr_subgrids < 0) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids < 0");
    if (nr_subgrids > 0 && (!subgrids || !grid)) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL subgrids or grid");
    return IDG_OK;
}

// Device buffers of the host-buffer cycle, kept between calls.
struct CycleBuffers {
    int device = -1;
    void *uvw = nullptr, *k = nullptr, *taper = nullptr, *aterms = nullptr, *md = nullptr;
    void *vis_in = nullptr, *vis_out = nullptr, *subgrids = nullptr, *grid = nullptr;
    void *uvw2 = nullptr, *md2 = nullptr; // the odd cycles' plan and uvw in a call of several cycles
    size_t b_uvw = 0, b_k = 0, b_taper = 0, b_aterms = 0, b_md = 0, b_vis = 0, b_vis_out = 0, b_sub = 0, b_grid = 0;
    size_t b_uvw2 = 0, b_md2 = 0;
    cudaStream_t s_compute = nullptr, s_h2d = nullptr, s_d2h = nullptr;
    double next_ratio = 1.6; // IDG_CHUNKS_ADAPTIVE: the ratio the next call uses

    void release() {
        for (void *p : {uvw, k, taper, aterms, md, vis_in, vis_out, subgrids, grid, uvw2, md2})
            if (p) cudaFree(p);
        uvw = k = taper = aterms = md = vis_in = vis_out = subgrids = grid = uvw2 = md2 = nullptr;
        b_uvw = b_k = b_taper = b_aterms = b_md = b_vis = b_vis_out = b_sub = b_grid = b_uvw2 = b_md2 = 0;
        for (cudaStream_t s : {s_compute, s_h2d, s_d2h})
            if (s) cudaStreamDestroy(s);
        s_compute = s_h2d = s_d2h = nullptr;
        device = -1;
    }
};
std::mutex g_cycle_mutex;
CycleBuffers g_cycle;

// A chunk of the host-buffer cycle: subgrids [s0, s1) and the rows [r0, r1)
// they name.
struct Chunk {
    int64_t s0, s1, r0, r1;
};

// Subgrid boundaries 0 = b0 < b1 < ... = n.  chunk > 0: equal chunks of that
// many subgrids; IDG_CHUNKS_AUTO / IDG_CHUNKS_ADAPTIVE: `pieces` chunks
// whose sizes grow by `ratio` from one to the next (`growing`) or shrink by
// it (otherwise), chunks under kMinChunk subgrids merged into their
// neighbour; anything else: one chunk.  A growing chunk's copy keeps ahead of
// the previous chunk's kernels while the copy rate is at least `ratio` times
// the rate the kernels consume visibilities (about 61 GB/s for the config-2
// gridder: at ratio 1.6, copies at 98 GB/s or more suffice).
constexpr int64_t kMinChunk = 1024;
constexpr int kAutoChunks = 10;
constexpr int kRunChunks = 4; // see run_cycles
constexpr double kAutoRatio = 1.6;
constexpr double kMinRatio = 1.1;
std::vector<int64_t> chunk_bounds(int64_t n, int64_t chunk, bool growing, double ratio, int pieces) {
    std::vector<int64_t> b{0};
    if (chunk == IDG_CHUNKS_AUTO || chunk == IDG_CHUNKS_ADAPTIVE) {
        const int k = pieces;
        double total = 0;
        for (int i = 0; i < k; ++i) total += std::pow(ratio, i);
        double acc = 0;
        for (int i = 0; i < k; ++i) {
            acc += std::pow(ratio, growing ? i : k - 1 - i);
            const int64_t e = i == k - 1 ? n : (int64_t)(n * acc / total + 0.5);
            if (e - b.back() >= kMinChunk) b.push_back(e);
        }
        if (b.size() == 1) b.push_back(n);
        b.back() = n; // the last chunk takes what the merges left
        return b;
    }
    if (chunk < 1 || chunk >= n) chunk = n;
    for (int64_t s = chunk; s < n; s += chunk) b.push_back(s);
    b.push_back(n);
    return b;
}

// The chunks of `bounds` with their row ranges; false when a chunk's rows
// start before the previous chunk's end (the plan is not in row order).
bool make_chunks(const std::vector<int64_t> &bounds, const std::vector<int64_t> &row0,
                 const std::vector<int64_t> &row1, std::vector<Chunk> *out) {
    out->clear();
    int64_t prev_end = 0;
    for (size_t i = 0; i + 1 < bounds.size(); ++i) {
        Chunk c{bounds[i], bounds[i + 1], INT64_MAX, 0};
        for (int64_t s = c.s0; s < c.s1; ++s) {
            c.r0 = std::min(c.r0, row0[s]);
            c.r1 = std::max(c.r1, row1[s]);
        }
        if (c.r0 < prev_end) return false;
        prev_end = c.r1;
        out->push_back(c);
    }
    return true;
}

int ensure(void **p, size_t *have, size_t want) {
    if (want == 0) want = 16;
    if (*p && *have >= want) return IDG_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    IDG_CUDA(cudaMalloc(p, want));
    *have = want;
    return IDG_OK;
}

} // namespace

extern "C" {

IDG_API int idg_grid_visibilities(const idg_params *params, int variant, int64_t nr_subgrids,
                                  const idg_metadata *metadata, const idg_subgrid_ext *ext, int64_t nr_rows,
                                  const float *uvw, const float *wavenumbers, const void *visibilities,
                                  const float *spheroidal, const void *aterms, void *subgrids, void *grid,
                                  void *stream) {
    if (int rc = check_step_args(params, nr_subgrids, subgrids, grid)) return rc;
    if (nr_subgrids == 0) return IDG_OK;
    idg_params p = *params;
    p.flags |= IDG_FLAG_NO_TAPER;
    if (int rc = idg_gridder(&p, variant, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers, visibilities,
                             nullptr, aterms, subgrids, stream))
        return rc;
    if (int rc = idg_subgrid_fft(params, nr_subgrids, +1, spheroidal, subgrids, stream)) return rc;
    return idg_adder(params, nr_subgrids, metadata, subgrids, grid, stream);
}

IDG_API int idg_degrid_visibilities(const idg_params *params, int variant, int64_t nr_subgrids,
                                    const idg_metadata *metadata, const idg_subgrid_ext *ext, int64_t nr_rows,
                                    const float *uvw, const float *wavenumbers, void *visibilities,
                                    const float *spheroidal, const void *aterms, void *subgrids, const void *grid,
                                    void *stream) {
    if (int rc = check_step_args(params, nr_subgrids, subgrids, grid)) return rc;
    if (nr_subgrids == 0) return IDG_OK;
    if (!fft_size_supported(params->subgrid_size))
        return fail(IDG_ERR_UNSUPPORTED, "subgrid_size %d: the subgrid FFT supports 8, 16, 24, 32, 48, 64",
                    params->subgrid_size);
    if (!metadata) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (reinterpret_cast<uintptr_t>(subgrids) % 16 != 0)
        return fail(IDG_ERR_INVALID_ARGUMENT, "subgrids must be 16-byte aligned");
    // splitter and backward subgrid FFT in one pass
    cudaError_t e = launch_split_fft(metadata, nr_subgrids, params->subgrid_size, params->grid_size,
                                     params->nr_w_planes > 0 ? params->nr_w_planes : 1,
                                     static_cast<const float2 *>(grid), static_cast<float2 *>(subgrids), spheroidal,
                                     reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "split + subgrid fft launch");
    idg_params p = *params;
    p.flags |= IDG_FLAG_NO_TAPER;
    return idg_degridder(&p, variant, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers, visibilities, nullptr,
                         aterms, subgrids, stream);
}

IDG_API int idg_release_buffers(void) {
    std::lock_guard<std::mutex> lock(g_cycle_mutex);
    g_cycle.release();
    return IDG_OK;
}

} // extern "C"

namespace {

// One cycle of a host-buffer call: the rows its entries name, its chunks, the
// device buffers of its plan and uvw, and the events that order it against
// the cycles either side and time it.
struct CycleRun {
    const idg_cycle_io *io = nullptr;
    std::vector<std::pair<int64_t, int64_t>> gaps; // rows no entry names
    std::vector<Chunk> gch, dch;
    void *md = nullptr, *uvw = nullptr;
    cudaEvent_t t_start, md_in, t_grid0, t_grid1, t_deg1, t_end;
    // per gridding chunk: its copy in bracketed on s_h2d (h2d_b, h2d_e), its
    // kernels started after the wait for it (g_go) and ended with its adder
    // (g_end); per degridding chunk: its kernels done, its copy out
    // bracketed on s_d2h
    std::vector<cudaEvent_t> h2d_b, h2d_e, g_go, g_end, deg_done, d2h_b, d2h_e;
    int64_t launches = 0, h2d = 0, d2h = 0, h2d_vis = 0, d2h_vis = 0;
};

// cycles of one idg_imaging_cycles call: each holds its own events (about
// 70 at ten chunks per phase), created before the first copy is queued
constexpr int kMaxCycles = 4096;

bool ranges_overlap(const void *a, size_t na, const void *b, size_t nb) {
    if (!a || !b || na == 0 || nb == 0) return false;
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + nb && y < x + na;
}

// The cycles of idg_imaging_cycle (one) and idg_imaging_cycles (several),
// enqueued on the three streams of the cycle buffers.  Cycle i+1's copies in
// start once cycle i's gridding has started (its plan and uvw go to the other
// one of two buffers, which cycle i-1 has finished with), each chunk's
// visibilities once cycle i's gridding chunks that read those rows have
// ended, so they run while cycle i grids and degrids.  Cycle i+1's degridding
// waits for cycle i's copies out (the visibilities out are one buffer), and
// its gridding for cycle i's grid copy when there is one.
int run_cycles(const idg_params *params, int variant, int64_t nr_cycles, const idg_cycle_io *io,
               const float *wavenumbers, const float *spheroidal, const void *aterms, int64_t chunk_subgrids,
               bool single) {
    if (int rc = check_params(params, true)) return rc;
    if (!single && (nr_cycles < 1 || nr_cycles > kMaxCycles || !io))
        return fail(IDG_ERR_INVALID_ARGUMENT, "nr_cycles outside [1, %d] or NULL cycles", kMaxCycles);
    const int64_t S = params->subgrid_size, C = params->nr_channels, G = params->grid_size;
    const int64_t W = params->nr_w_planes > 0 ? params->nr_w_planes : 1;
    const size_t row_bytes = (size_t)C * 32, b_grid = (size_t)W * 4 * G * G * 8;

    std::vector<CycleRun> runs(nr_cycles);
    std::vector<std::vector<int64_t>> row0(nr_cycles), row1(nr_cycles);
    int64_t max_sub = 0, max_rows = 0;
    for (int64_t i = 0; i < nr_cycles; ++i) {
        const idg_cycle_io &c = io[i];
        char tag[40] = "";
        if (!single) std::snprintf(tag, sizeof tag, "cycle %lld: ", (long long)i);
        if (c.nr_subgrids < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "%snr_subgrids < 1", tag);
        if (c.nr_rows < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "%snr_rows < 1", tag);
        if (!c.metadata || !c.uvw || !wavenumbers || !c.visibilities_in || !spheroidal || !aterms ||
            !c.visibilities_out)
            return fail(IDG_ERR_INVALID_ARGUMENT, "%sNULL host array", tag);
        // rows of every entry, checked; the chunks of each phase follow under
        // the lock (rows must advance chunk by chunk for the copies to
        // overlap the kernels)
        CycleRun &r = runs[i];
        r.io = &c;
        const int bo1 = c.metadata[0].baseline_offset;
        std::vector<int64_t> &a0 = row0[i], &a1 = row1[i];
        a0.resize(c.nr_subgrids);
        a1.resize(c.nr_subgrids);
        for (int64_t s = 0; s < c.nr_subgrids; ++s) {
            const idg_metadata &m = c.metadata[s];
            const int64_t a = (int64_t)(m.baseline_offset - bo1) + m.time_offset;
            if (a < 0 || m.nr_timesteps < 0 || a + m.nr_timesteps > c.nr_rows)
                return fail(IDG_ERR_INVALID_ARGUMENT, "%splan entry %lld names rows outside [0, %lld)", tag,
                            (long long)s, (long long)c.nr_rows);
            a0[s] = a;
            a1[s] = a + m.nr_timesteps;
        }
        // rows that no entry names (zeroed in the output instead of degridded)
        std::vector<std::pair<int64_t, int64_t>> spans(c.nr_subgrids);
        for (int64_t s = 0; s < c.nr_subgrids; ++s) spans[s] = {a0[s], a1[s]};
        std::sort(spans.begin(), spans.end());
        int64_t covered = 0;
        for (const auto &sp : spans) {
            if (sp.first > covered) r.gaps.push_back({covered, sp.first});
            covered = std::max(covered, sp.second);
        }
        if (covered < c.nr_rows) r.gaps.push_back({covered, c.nr_rows});
        max_sub = std::max(max_sub, c.nr_subgrids);
        max_rows = std::max(max_rows, c.nr_rows);
    }
    // A cycle's copies in start before the cycles ahead of it have copied
    // their results out: no cycle may read host memory an earlier one writes.
    for (int64_t i = 0; i < nr_cycles; ++i)
        for (int64_t j = i + 1; j < nr_cycles; ++j) {
            const idg_cycle_io &a = io[i], &b = io[j];
            const size_t out = (size_t)a.nr_rows * row_bytes;
            const void *writes[2] = {a.visibilities_out, a.grid_out};
            const size_t wn[2] = {out, a.grid_out ? b_grid : 0};
            const void *reads[3] = {b.visibilities_in, b.uvw, b.metadata};
            const size_t rn[3] = {(size_t)b.nr_rows * row_bytes, (size_t)b.nr_rows * 12,
                                  (size_t)b.nr_subgrids * sizeof(idg_metadata)};
            for (int x = 0; x < 2; ++x)
                for (int y = 0; y < 3; ++y)
                    if (ranges_overlap(writes[x], wn[x], reads[y], rn[y]))
                        return fail(IDG_ERR_INVALID_ARGUMENT,
                                    "cycle %lld reads host memory that cycle %lld writes: run them as separate "
                                    "calls",
                                    (long long)j, (long long)i);
        }

    std::lock_guard<std::mutex> lock(g_cycle_mutex);
    CycleBuffers &B = g_cycle;
    // the gridding phase's growth ratio (the degridding phase's copies out
    // have run at the full device-to-host rate on every host measured: it
    // keeps kAutoRatio)
    const double ratio = chunk_subgrids == IDG_CHUNKS_ADAPTIVE ? B.next_ratio : kAutoRatio;
    for (int64_t i = 0; i < nr_cycles; ++i) {
        CycleRun &r = runs[i];
        const int64_t n = r.io->nr_subgrids;
        // In a run of cycles, a cycle after the first finds most of its
        // visibilities on the device (copied while the cycle before it ran),
        // and a cycle before the last has until the next cycle's degridding to
        // copy its results out: kRunChunks chunks suffice there, with fewer
        // partial last waves of the persistent kernels.  The first cycle's
        // gridding and the last cycle's degridding keep kAutoChunks.
        const int gp = i == 0 ? kAutoChunks : kRunChunks, dp = i + 1 == nr_cycles ? kAutoChunks : kRunChunks;
        if (!make_chunks(chunk_bounds(n, chunk_subgrids, true, i == 0 ? ratio : kAutoRatio, gp), row0[i], row1[i],
                         &r.gch) ||
            !make_chunks(chunk_bounds(n, chunk_subgrids, false, kAutoRatio, dp), row0[i], row1[i], &r.dch)) {
            r.gch.assign(1, Chunk{0, n, 0, r.io->nr_rows});
            r.dch = r.gch;
        }
    }
    int dev = 0;
    IDG_CUDA(cudaGetDevice(&dev));
    if (B.device != dev) {
        B.release();
        B.device = dev;
    }
    if (!B.s_compute) {
        IDG_CUDA(cudaStreamCreateWithFlags(&B.s_compute, cudaStreamNonBlocking));
        IDG_CUDA(cudaStreamCreateWithFlags(&B.s_h2d, cudaStreamNonBlocking));
        IDG_CUDA(cudaStreamCreateWithFlags(&B.s_d2h, cudaStreamNonBlocking));
    }
    const size_t b_uvw = (size_t)max_rows * 12, b_k = (size_t)C * 4, b_taper = (size_t)S * S * 4,
                 b_aterms = (size_t)params->nr_aterms * params->nr_stations * S * S * 32,
                 b_md = (size_t)max_sub * sizeof(idg_metadata), b_vis = (size_t)max_rows * row_bytes,
                 b_sub = (size_t)max_sub * 4 * S * S * 8;
    if (int rc = ensure(&B.uvw, &B.b_uvw, b_uvw)) return rc;
    if (int rc = ensure(&B.k, &B.b_k, b_k)) return rc;
    if (int rc = ensure(&B.taper, &B.b_taper, b_taper)) return rc;
    if (int rc = ensure(&B.aterms, &B.b_aterms, b_aterms)) return rc;
    if (int rc = ensure(&B.md, &B.b_md, b_md)) return rc;
    if (int rc = ensure(&B.vis_in, &B.b_vis, b_vis)) return rc;
    if (int rc = ensure(&B.vis_out, &B.b_vis_out, b_vis)) return rc;
    if (int rc = ensure(&B.subgrids, &B.b_sub, b_sub)) return rc;
    if (int rc = ensure(&B.grid, &B.b_grid, b_grid)) return rc;
    if (nr_cycles > 1) {
        if (int rc = ensure(&B.uvw2, &B.b_uvw2, b_uvw)) return rc;
        if (int rc = ensure(&B.md2, &B.b_md2, b_md)) return rc;
    }
    for (int64_t i = 0; i < nr_cycles; ++i) {
        runs[i].md = i % 2 ? B.md2 : B.md;
        runs[i].uvw = i % 2 ? B.uvw2 : B.uvw;
    }

    std::vector<cudaEvent_t> ev;
    auto new_event = [&](cudaEvent_t *e, bool timing_event) -> int {
        IDG_CUDA(cudaEventCreateWithFlags(e, timing_event ? cudaEventDefault : cudaEventDisableTiming));
        ev.push_back(*e);
        return IDG_OK;
    };
    struct EventGuard {
        std::vector<cudaEvent_t> &v;
        ~EventGuard() {
            for (cudaEvent_t e : v) cudaEventDestroy(e);
        }
    } guard{ev};
    for (CycleRun &r : runs) {
        for (cudaEvent_t *e : {&r.t_start, &r.t_grid0, &r.t_grid1, &r.t_deg1, &r.t_end})
            if (int rc = new_event(e, true)) return rc;
        if (int rc = new_event(&r.md_in, false)) return rc;
        const size_t ng = r.gch.size(), nd = r.dch.size();
        r.h2d_b.resize(ng);
        r.h2d_e.resize(ng);
        r.g_go.resize(ng);
        r.g_end.resize(ng);
        r.deg_done.resize(nd);
        r.d2h_b.resize(nd);
        r.d2h_e.resize(nd);
        for (size_t i = 0; i < ng; ++i) {
            if (int rc = new_event(&r.h2d_b[i], true)) return rc;
            if (int rc = new_event(&r.h2d_e[i], true)) return rc;
            if (int rc = new_event(&r.g_go[i], true)) return rc;
            if (int rc = new_event(&r.g_end[i], true)) return rc;
        }
        for (size_t i = 0; i < nd; ++i) {
            if (int rc = new_event(&r.deg_done[i], false)) return rc;
            if (int rc = new_event(&r.d2h_b[i], true)) return rc;
            if (int rc = new_event(&r.d2h_e[i], true)) return rc;
        }
    }

    DeviceWords w;
    if (int rc = device_words(&w)) return rc;
    IDG_CUDA(cudaDeviceSynchronize());
    // From here on every return -- early ones included -- first waits for the
    // call's streams, so that no copy from or into the caller's host buffers
    // is still queued when the call returns.  (Declared after the event guard,
    // so it runs before the events are destroyed.)
    struct StreamGuard {
        cudaStream_t s[3];
        ~StreamGuard() {
            for (cudaStream_t x : s) cudaStreamSynchronize(x);
        }
    } stream_guard{{B.s_h2d, B.s_compute, B.s_d2h}};
    // The check word is library-wide: clear what earlier, unrelated calls left
    // in it, so that the status read at the end is this call's own.
    IDG_CUDA(cudaMemsetAsync(w.status, 0, sizeof(unsigned), B.s_compute));

    for (int64_t ci = 0; ci < nr_cycles; ++ci) {
        CycleRun &r = runs[ci];
        const CycleRun *prev = ci > 0 ? &runs[ci - 1] : nullptr;
        const idg_cycle_io &c = *r.io;
        const int64_t nr_rows = c.nr_rows;
        // copies in: the constants once, before the first plan; a later
        // cycle's after the previous cycle's gridding has started, and each
        // chunk's visibilities after the previous cycle's gridding chunks
        // that read the rows they overwrite
        if (prev) IDG_CUDA(cudaStreamWaitEvent(B.s_h2d, prev->t_grid0, 0));
        IDG_CUDA(cudaEventRecord(r.t_start, B.s_h2d));
        if (!prev) {
            IDG_CUDA(cudaMemcpyAsync(B.k, wavenumbers, b_k, cudaMemcpyHostToDevice, B.s_h2d));
            IDG_CUDA(cudaMemcpyAsync(B.taper, spheroidal, b_taper, cudaMemcpyHostToDevice, B.s_h2d));
            IDG_CUDA(cudaMemcpyAsync(B.aterms, aterms, b_aterms, cudaMemcpyHostToDevice, B.s_h2d));
            r.h2d += b_k + b_taper + b_aterms;
        }
        const size_t md_bytes = (size_t)c.nr_subgrids * sizeof(idg_metadata);
        IDG_CUDA(cudaMemcpyAsync(r.md, c.metadata, md_bytes, cudaMemcpyHostToDevice, B.s_h2d));
        r.h2d += md_bytes;
        IDG_CUDA(cudaEventRecord(r.md_in, B.s_h2d));
        int64_t waited = -1; // the previous cycle's last gridding chunk waited for
        for (size_t i = 0; i < r.gch.size(); ++i) {
            const Chunk &k = r.gch[i];
            // uvw: this chunk's rows, with any rows before them that no chunk
            // names (and, for the last chunk, the rows after it)
            const int64_t u0 = i == 0 ? 0 : r.gch[i - 1].r1, u1 = i + 1 == r.gch.size() ? nr_rows : k.r1;
            if (u1 > u0) {
                IDG_CUDA(cudaMemcpyAsync(static_cast<char *>(r.uvw) + (size_t)u0 * 12,
                                         reinterpret_cast<const char *>(c.uvw) + (size_t)u0 * 12,
                                         (size_t)(u1 - u0) * 12, cudaMemcpyHostToDevice, B.s_h2d));
                r.h2d += (u1 - u0) * 12;
            }
            if (prev) {
                // the previous cycle's chunks are in row order: the last one
                // starting before this chunk's rows end is the last reader
                int64_t last = -1;
                for (size_t q = 0; q < prev->gch.size() && prev->gch[q].r0 < k.r1; ++q) last = (int64_t)q;
                if (last > waited) {
                    IDG_CUDA(cudaStreamWaitEvent(B.s_h2d, prev->g_end[last], 0));
                    waited = last;
                }
            }
            const size_t off = (size_t)k.r0 * row_bytes, bytes = (size_t)(k.r1 - k.r0) * row_bytes;
            IDG_CUDA(cudaEventRecord(r.h2d_b[i], B.s_h2d));
            IDG_CUDA(cudaMemcpyAsync(static_cast<char *>(B.vis_in) + off,
                                     static_cast<const char *>(c.visibilities_in) + off, bytes,
                                     cudaMemcpyHostToDevice, B.s_h2d));
            IDG_CUDA(cudaEventRecord(r.h2d_e[i], B.s_h2d));
            r.h2d += bytes;
            r.h2d_vis += bytes;
        }

        // gridding phase (after the previous cycle's grid copy, if any: the
        // grid is zeroed here)
        IDG_CUDA(cudaStreamWaitEvent(B.s_compute, r.md_in, 0));
        if (prev && prev->io->grid_out) IDG_CUDA(cudaStreamWaitEvent(B.s_compute, prev->t_end, 0));
        IDG_CUDA(cudaMemsetAsync(B.grid, 0, b_grid, B.s_compute));
        IDG_CUDA(cudaEventRecord(r.t_grid0, B.s_compute));
        const idg_metadata *d_md = static_cast<const idg_metadata *>(r.md);
        for (size_t i = 0; i < r.gch.size(); ++i) {
            IDG_CUDA(cudaStreamWaitEvent(B.s_compute, r.h2d_e[i], 0));
            IDG_CUDA(cudaEventRecord(r.g_go[i], B.s_compute));
            const int64_t s0 = r.gch[i].s0, n = r.gch[i].s1 - s0;
            if (int rc = idg_grid_visibilities(params, variant, n, d_md + s0, nullptr, nr_rows,
                                               (const float *)r.uvw, (const float *)B.k, B.vis_in,
                                               (const float *)B.taper, B.aterms,
                                               static_cast<char *>(B.subgrids) + (size_t)s0 * 4 * S * S * 8, B.grid,
                                               B.s_compute))
                return rc;
            r.launches += 3;
            IDG_CUDA(cudaEventRecord(r.g_end[i], B.s_compute));
        }
        IDG_CUDA(cudaEventRecord(r.t_grid1, B.s_compute));

        // degridding phase, after the previous cycle's copies out: the
        // degridder writes every row a plan entry names; the rows no entry
        // names come back as zeros
        if (prev) IDG_CUDA(cudaStreamWaitEvent(B.s_compute, prev->t_end, 0));
        for (const auto &gap : r.gaps)
            IDG_CUDA(cudaMemsetAsync(static_cast<char *>(B.vis_out) + (size_t)gap.first * row_bytes, 0,
                                     (size_t)(gap.second - gap.first) * row_bytes, B.s_compute));
        for (size_t i = 0; i < r.dch.size(); ++i) {
            const int64_t s0 = r.dch[i].s0, n = r.dch[i].s1 - s0;
            if (int rc = idg_degrid_visibilities(params, variant, n, d_md + s0, nullptr, nr_rows,
                                                 (const float *)r.uvw, (const float *)B.k, B.vis_out,
                                                 (const float *)B.taper, B.aterms,
                                                 static_cast<char *>(B.subgrids) + (size_t)s0 * 4 * S * S * 8, B.grid,
                                                 B.s_compute))
                return rc;
            r.launches += 3;
            IDG_CUDA(cudaEventRecord(r.deg_done[i], B.s_compute));
            IDG_CUDA(cudaStreamWaitEvent(B.s_d2h, r.deg_done[i], 0));
            // this chunk's rows, with the rows before them that no chunk names
            // (and, for the last chunk, the rows after it): zeroed above
            const int64_t v0 = i == 0 ? 0 : r.dch[i - 1].r1, v1 = i + 1 == r.dch.size() ? nr_rows : r.dch[i].r1;
            const size_t off = (size_t)v0 * row_bytes, bytes = (size_t)(v1 - v0) * row_bytes;
            IDG_CUDA(cudaEventRecord(r.d2h_b[i], B.s_d2h));
            IDG_CUDA(cudaMemcpyAsync(static_cast<char *>(c.visibilities_out) + off,
                                     static_cast<char *>(B.vis_out) + off, bytes, cudaMemcpyDeviceToHost, B.s_d2h));
            IDG_CUDA(cudaEventRecord(r.d2h_e[i], B.s_d2h));
            r.d2h += bytes;
            r.d2h_vis += bytes;
        }
        IDG_CUDA(cudaEventRecord(r.t_deg1, B.s_compute));
        if (c.grid_out) {
            IDG_CUDA(cudaStreamWaitEvent(B.s_d2h, r.t_grid1, 0));
            IDG_CUDA(cudaMemcpyAsync(c.grid_out, B.grid, b_grid, cudaMemcpyDeviceToHost, B.s_d2h));
            r.d2h += b_grid;
        }
        IDG_CUDA(cudaEventRecord(r.t_end, B.s_d2h));
    }
    IDG_CUDA(cudaEventSynchronize(runs.back().t_end));
    IDG_CUDA(cudaStreamSynchronize(B.s_compute));

    unsigned status = 0;
    IDG_CUDA(cudaMemcpy(&status, w.status, sizeof status, cudaMemcpyDeviceToHost));
    if (status) {
        IDG_CUDA(cudaMemset(w.status, 0, sizeof(unsigned)));
        return fail(IDG_ERR_DEVICE_CHECK, "a kernel rejected plan entries (status 0x%x)", status);
    }
    for (int64_t ci = 0; ci < nr_cycles; ++ci) {
        const CycleRun &r = runs[ci];
        float total = 0, g = 0, d = 0, end = 0, span = 0;
        IDG_CUDA(cudaEventElapsedTime(&total, r.t_start, r.t_end));
        IDG_CUDA(cudaEventElapsedTime(&span, r.t_start, r.h2d_e.back()));
        IDG_CUDA(cudaEventElapsedTime(&end, runs[0].t_start, r.t_end));
        IDG_CUDA(cudaEventElapsedTime(&g, r.t_grid0, r.t_grid1));
        IDG_CUDA(cudaEventElapsedTime(&d, r.t_grid1, r.t_deg1));
        double hv = 0; // the visibility copies in alone
        for (size_t i = 0; i < r.gch.size(); ++i) {
            float x = 0;
            IDG_CUDA(cudaEventElapsedTime(&x, r.h2d_b[i], r.h2d_e[i]));
            hv += x;
        }
        // the gridding kernels' waits for their copies: before the first chunk
        // (after the grid was zeroed) and between one chunk's end and the next's start
        double wait = 0;
        for (size_t i = 0; i < r.gch.size(); ++i) {
            float x = 0;
            IDG_CUDA(cudaEventElapsedTime(&x, i == 0 ? r.t_grid0 : r.g_end[i - 1], r.g_go[i]));
            wait += x;
        }
        if (ci == 0 && chunk_subgrids == IDG_CHUNKS_ADAPTIVE && r.gch.size() > 1 && hv > 0 && g - wait > 0) {
            // next call: at most 0.9 x (copy rate / kernel rate), the largest
            // ratio whose growing copies still end before their kernels are
            // due at the average copy rate; copies arrive unevenly, so a cycle
            // whose kernels waited more than 2 % of the phase also steps the
            // ratio down by 15 %, and one that did not lets it grow back by
            // 5 %.  Only the call's first cycle counts: the copies of the
            // cycles after it ran ahead, during the degridding before them.
            const double by_rate = 0.9 * (g - wait) / hv;
            const double by_wait = ratio * (wait > 0.02 * g ? 0.85 : 1.05);
            B.next_ratio = std::min(kAutoRatio, std::max(kMinRatio, std::min(by_rate, by_wait)));
        }
        idg_cycle_timing *timing = r.io->timing;
        if (!timing) continue;
        timing->total_ms = total;
        timing->gridding_ms = g;
        timing->degridding_ms = d;
        timing->h2d_bytes = r.h2d;
        timing->d2h_bytes = r.d2h;
        timing->kernel_launches = r.launches;
        double dv = 0;
        for (size_t i = 0; i < r.dch.size(); ++i) {
            float x = 0;
            IDG_CUDA(cudaEventElapsedTime(&x, r.d2h_b[i], r.d2h_e[i]));
            dv += x;
        }
        timing->h2d_vis_ms = hv;
        timing->d2h_vis_ms = dv;
        timing->h2d_vis_bytes = r.h2d_vis;
        timing->d2h_vis_bytes = r.d2h_vis;
        timing->grid_chunks = (int64_t)r.gch.size();
        timing->degrid_chunks = (int64_t)r.dch.size();
        timing->gridding_wait_ms = wait;
        timing->chunk_ratio =
            (chunk_subgrids == IDG_CHUNKS_AUTO || chunk_subgrids == IDG_CHUNKS_ADAPTIVE) ? ratio : 0.0;
        timing->end_ms = end;
        timing->h2d_span_ms = span;
    }
    return IDG_OK;
}

} // namespace

extern "C" {

IDG_API int idg_imaging_cycle(const idg_params *params, int variant, int64_t nr_subgrids,
                              const idg_metadata *metadata, int64_t nr_rows, const float *uvw,
                              const float *wavenumbers, const void *visibilities_in, const float *spheroidal,
                              const void *aterms, void *visibilities_out, void *grid_out, int64_t chunk_subgrids,
                              idg_cycle_timing *timing) {
    const idg_cycle_io io{nr_subgrids, metadata, nr_rows, uvw, visibilities_in, visibilities_out, grid_out, timing};
    return run_cycles(params, variant, 1, &io, wavenumbers, spheroidal, aterms, chunk_subgrids, true);
}

IDG_API int idg_imaging_cycles(const idg_params *params, int variant, int64_t nr_cycles, const idg_cycle_io *cycles,
                               const float *wavenumbers, const float *spheroidal, const void *aterms,
                               int64_t chunk_subgrids) {
    return run_cycles(params, variant, nr_cycles, cycles, wavenumbers, spheroidal, aterms, chunk_subgrids, false);
}

} // extern "C"
