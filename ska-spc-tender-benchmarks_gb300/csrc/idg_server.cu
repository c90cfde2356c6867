// idg_server.cu -- the serving loop: continuous batching of gridding and
// degridding jobs on one GPU.
//
// Jobs arrive on any thread through idg_server_submit().  A scheduler thread
// admits them in arrival order whenever a slot (a CUDA stream) is free and the
// job's device footprint fits the HBM budget left by the jobs already running
// -- a job that can never fit is rejected at submission.  An admitted job gets
// one stream-ordered allocation for its plan, subgrid work space and data, its
// copies in, the batched kernels of its step and its copies out, all on its
// slot's stream; so jobs that are admitted while others run overlap on the
// device (copies against kernels, and kernels against kernels when the
// persistent kernels' CTA budget is shared between the running jobs).  uv-grids
// live on the device for the server's lifetime: gridding jobs add into one,
// degridding jobs read one; a job whose kind differs from the running jobs on
// the same grid waits for them on the GPU (stream-ordered event waits).  The
// adder sums in a fixed order (tile bins made on the host at submission,
// idg_tiles.cu), and the adders of gridding jobs on one grid run one after
// another in admission order, so a grid's contents do not depend on how the
// jobs overlapped.  The scheduler polls completion (never blocks in a CUDA
// call), records queueing, run and total latency per job, and frees the job's
// memory.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"
#include "idg_tiles.h"

using namespace idg;
using Clock = std::chrono::steady_clock;

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Grid {
    void *dev = nullptr;
    size_t bytes = 0;
    int32_t size = 0, planes = 1;
    int last_op = -1;                  // op of the jobs currently holding the grid
    std::vector<cudaEvent_t> holders;  // their completion events
    int readers = 0;                   // idg_server_grid_read calls copying the grid out
    cudaEvent_t last_add = nullptr;    // end of the adder of the last gridding job admitted on it
};

struct Job {
    int64_t id = 0;
    idg_job spec{};
    std::vector<idg_metadata> md;
    std::vector<idg_subgrid_ext> ext;
    std::vector<int> work;
    size_t footprint = 0;
    int64_t nvis = 0;
    Clock::time_point t_submit, t_admit, t_done;
    int slot = -1;
    void *arena = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t k0 = nullptr, k1 = nullptr; // around the job's kernels (timing events)
    cudaEvent_t c0 = nullptr, c1 = nullptr; // around all of its stream work, copies included
    cudaEvent_t add_done = nullptr;         // gridding jobs: after the adder
    TileBinsHost bins;                      // gridding jobs: the adder's tile bins
    double dev_start_ms = -1, dev_end_ms = -1; // k0, k1 relative to the server's epoch event
    double work_start_ms = -1, work_end_ms = -1; // c0, c1
    double est_ms = 0;                      // estimated device time at the full CTA budget
    int share = 1;                          // its kernels' share of that budget: 1 / share
    int status = IDG_OK;
    bool finished = false;
};

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
    size_t md, ext, work, words, sub, uvw, k, taper, aterms, vis, entries, items, multi, partials, total;
};

Layout job_layout(const idg_job &j, const TileBinsHost *bins = nullptr) {
    const idg_params &p = j.params;
    const size_t N = (size_t)j.nr_subgrids, S = (size_t)p.subgrid_size;
    Layout L;
    size_t off = 0;
    L.md = off; off += align_up(sizeof(idg_metadata) * N);
    L.ext = off; off += j.ext ? align_up(sizeof(idg_subgrid_ext) * N) : 0;
    L.work = off; off += align_up(sizeof(int) * N);
    L.words = off; off += 256;
    L.sub = off; off += align_up(N * 4 * S * S * 8);
    L.uvw = off; off += align_up((size_t)j.nr_rows * 12);
    L.k = off; off += align_up((size_t)p.nr_channels * 4);
    L.taper = off; off += align_up(S * S * 4);
    L.aterms = off; off += align_up((size_t)p.nr_aterms * p.nr_stations * S * S * 32);
    L.vis = off; off += align_up((size_t)j.nr_rows * p.nr_channels * 32);
    L.entries = off; off += bins ? align_up(sizeof(int) * bins->entries.size()) : 0;
    L.items = off; off += bins ? align_up(sizeof(TileItem) * bins->items.size()) : 0;
    L.multi = off; off += bins ? align_up(sizeof(TileMulti) * bins->multi.size()) : 0;
    L.partials = off; off += bins ? align_up(bins->partial_bytes()) : 0;
    L.total = off;
    return L;
}

} // namespace

struct idg_server {
    idg_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Job>> queue;
    std::map<int64_t, std::shared_ptr<Job>> jobs;
    std::vector<std::shared_ptr<Job>> slots;
    std::vector<cudaStream_t> streams;
    cudaEvent_t epoch = nullptr; // recorded at creation: origin of the jobs' device intervals
    std::map<int64_t, Grid> grids;
    int64_t next_job = 1, next_grid = 1;
    size_t in_use = 0, peak_use = 0;
    // device milliseconds per 1e9 pixel-visibilities of a job's kernels at the
    // full CTA budget: a running estimate from the finished jobs (seeded with
    // GB300's config-2 rate)
    double ms_per_gpv = 0.6;
    int64_t completed = 0, rejected = 0, failed = 0, total_vis = 0;
    std::vector<double> latencies;
    Clock::time_point first_submit{}, last_done{};
    bool have_first = false;
    bool stop = false;
    std::thread worker;

    void run();
    void admit_locked();
    void launch(Job &j);
    void poll_locked();
};

namespace {

int validate_job(const idg_server *srv, const idg_job *j) {
    if (!j) return fail(IDG_ERR_INVALID_ARGUMENT, "job is NULL");
    if (j->op != IDG_JOB_GRID && j->op != IDG_JOB_DEGRID) return fail(IDG_ERR_INVALID_ARGUMENT, "unknown job op %d", j->op);
    if (int rc = check_params(&j->params, true)) return rc;
    if (j->nr_subgrids < 1 || j->nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids");
    if (j->nr_rows < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_rows");
    if (!j->metadata || !j->uvw || !j->wavenumbers || !j->spheroidal || !j->aterms)
        return fail(IDG_ERR_INVALID_ARGUMENT, "NULL host array");
    if (j->op == IDG_JOB_GRID && !j->vis_in) return fail(IDG_ERR_INVALID_ARGUMENT, "gridding job without vis_in");
    if (j->op == IDG_JOB_DEGRID && !j->vis_out) return fail(IDG_ERR_INVALID_ARGUMENT, "degridding job without vis_out");
    auto it = srv->grids.find(j->grid_id);
    if (it == srv->grids.end()) return fail(IDG_ERR_NOT_FOUND, "unknown grid %lld", (long long)j->grid_id);
    if (it->second.size != j->params.grid_size || it->second.planes != (j->params.nr_w_planes > 0 ? j->params.nr_w_planes : 1))
        return fail(IDG_ERR_INVALID_ARGUMENT, "job geometry does not match grid %lld", (long long)j->grid_id);
    const int bo1 = j->metadata[0].baseline_offset;
    for (int64_t s = 0; s < j->nr_subgrids; ++s) {
        const idg_metadata &m = j->metadata[s];
        const int64_t r0 = (int64_t)(m.baseline_offset - bo1) + m.time_offset;
        int c0 = 0, c1 = j->params.nr_channels;
        if (j->ext) {
            c0 = j->ext[s].channel_begin;
            c1 = j->ext[s].channel_end;
        }
        if (r0 < 0 || m.nr_timesteps < 0 || r0 + m.nr_timesteps > j->nr_rows ||
            m.station1 >= (uint32_t)j->params.nr_stations || m.station2 >= (uint32_t)j->params.nr_stations ||
            m.aterm_index < 0 || m.aterm_index >= j->params.nr_aterms || c0 < 0 || c1 > j->params.nr_channels || c0 > c1)
            return fail(IDG_ERR_INVALID_ARGUMENT, "job plan entry %lld is out of range", (long long)s);
    }
    return IDG_OK;
}

} // namespace

void idg_server::launch(Job &j) {
    cudaSetDevice(device);
    cudaStream_t st = streams[j.slot];
    const idg_params &p = j.spec.params;
    const bool gridding = j.spec.op == IDG_JOB_GRID;
    const Layout L = job_layout(j.spec, gridding ? &j.bins : nullptr);
    char *base = static_cast<char *>(j.arena);
    auto dp = [&](size_t off) { return static_cast<void *>(base + off); };
    const size_t N = j.md.size();
    const int64_t S = p.subgrid_size;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess && x != cudaSuccess) e = x;
    };
    if (j.c0) chk(cudaEventRecord(j.c0, st));
    chk(cudaMemcpyAsync(dp(L.md), j.md.data(), sizeof(idg_metadata) * N, cudaMemcpyHostToDevice, st));
    if (!j.ext.empty()) chk(cudaMemcpyAsync(dp(L.ext), j.ext.data(), sizeof(idg_subgrid_ext) * N, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(dp(L.work), j.work.data(), sizeof(int) * N, cudaMemcpyHostToDevice, st));
    chk(cudaMemsetAsync(dp(L.words), 0, 256, st));
    chk(cudaMemcpyAsync(dp(L.uvw), j.spec.uvw, (size_t)j.spec.nr_rows * 12, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(dp(L.k), j.spec.wavenumbers, (size_t)p.nr_channels * 4, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(dp(L.taper), j.spec.spheroidal, (size_t)S * S * 4, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(dp(L.aterms), j.spec.aterms, (size_t)p.nr_aterms * p.nr_stations * S * S * 32,
                        cudaMemcpyHostToDevice, st));
    const size_t b_vis = (size_t)j.spec.nr_rows * p.nr_channels * 32;
    if (gridding) {
        chk(cudaMemcpyAsync(dp(L.vis), j.spec.vis_in, b_vis, cudaMemcpyHostToDevice, st));
        chk(cudaMemcpyAsync(dp(L.entries), j.bins.entries.data(), sizeof(int) * j.bins.entries.size(),
                            cudaMemcpyHostToDevice, st));
        if (!j.bins.items.empty())
            chk(cudaMemcpyAsync(dp(L.items), j.bins.items.data(), sizeof(TileItem) * j.bins.items.size(),
                                cudaMemcpyHostToDevice, st));
        if (!j.bins.multi.empty())
            chk(cudaMemcpyAsync(dp(L.multi), j.bins.multi.data(), sizeof(TileMulti) * j.bins.multi.size(),
                                cudaMemcpyHostToDevice, st));
    } else {
        chk(cudaMemsetAsync(dp(L.vis), 0, b_vis, st));
    }

    Grid &g = grids[j.spec.grid_id];
    KernelArgs a{};
    a.G = p.grid_size;
    a.S = p.subgrid_size;
    a.C = p.nr_channels;
    a.nr_stations = p.nr_stations;
    a.nr_aterms = p.nr_aterms;
    a.nr_w_planes = g.planes;
    a.image_size = p.image_size;
    a.w_step = p.w_step;
    a.flags = p.flags | IDG_FLAG_NO_TAPER;
    a.nr_subgrids = (int64_t)N;
    a.nr_rows = j.spec.nr_rows;
    a.md = static_cast<const idg_metadata *>(dp(L.md));
    a.ext = j.ext.empty() ? nullptr : static_cast<const idg_subgrid_ext *>(dp(L.ext));
    a.uvw = static_cast<const float *>(dp(L.uvw));
    a.wavenumbers = static_cast<const float *>(dp(L.k));
    a.taper = static_cast<const float *>(dp(L.taper));
    a.aterms = static_cast<const float4 *>(dp(L.aterms));
    a.vis = static_cast<float4 *>(dp(L.vis));
    a.subgrids = static_cast<float2 *>(dp(L.sub));
    a.work_list = static_cast<const int *>(dp(L.work));
    a.work_counter = static_cast<int *>(dp(L.words));
    a.status = static_cast<unsigned *>(dp(L.words)) + 2;
    // Running jobs share the SMs: a persistent kernel takes 1/share of the
    // CTAs that would fill the GPU with its own launch shape, and keeps them
    // to its end.  Peers estimated to finish within a quarter of this job's
    // own time do not count: the CTAs they free are this job's soon after.
    const double pixvis = (double)j.nvis * (double)p.subgrid_size * (double)p.subgrid_size;
    j.est_ms = pixvis * 1e-9 * ms_per_gpv;
    int share = 1;
    const Clock::time_point now = Clock::now();
    for (auto &other : slots) {
        if (!other || other.get() == &j) continue;
        const double left = other->est_ms * other->share - ms_between(other->t_admit, now);
        if (left > 0.25 * j.est_ms) ++share;
    }
    j.share = cfg.cta_share ? share : 1;
    a.share_den = j.share > 1 ? j.share : 0;
    const int variant = j.spec.variant == IDG_VARIANT_PLAIN ? IDG_VARIANT_PLAIN : IDG_VARIANT_BATCHED;

    // order against the other jobs on this grid
    if (g.last_op != -1 && g.last_op != j.spec.op)
        for (cudaEvent_t h : g.holders) chk(cudaStreamWaitEvent(st, h, 0));

    if (j.k0) chk(cudaEventRecord(j.k0, st));
    if (j.spec.op == IDG_JOB_GRID) {
        chk(launch_gridder(a, variant, p.nr_channels, st));
        chk(launch_subgrid_fft(a.subgrids, (int64_t)N, p.subgrid_size, +1, a.taper, st));
        // adders on one grid in admission order: this one after the previous one
        if (g.last_add) chk(cudaStreamWaitEvent(st, g.last_add, 0));
        TileBinsDev v;
        v.md = a.md;
        v.entries = static_cast<const int *>(dp(L.entries));
        v.items = static_cast<const TileItem *>(dp(L.items));
        v.multi = static_cast<const TileMulti *>(dp(L.multi));
        v.partials = j.bins.nslots ? static_cast<float2 *>(dp(L.partials)) : nullptr;
        v.S = j.bins.S;
        v.G = j.bins.G;
        v.ntx = j.bins.ntx;
        v.nitems = (int)j.bins.items.size();
        v.nmulti = (int)j.bins.multi.size();
        chk(launch_binned_adder(v, a.subgrids, static_cast<float2 *>(g.dev), st));
        // the next gridding job's adder waits for this one (for the whole job
        // when the event could not be made: j.done is recorded below)
        if (j.add_done) chk(cudaEventRecord(j.add_done, st));
        g.last_add = j.add_done ? j.add_done : j.done;
    } else {
        chk(launch_split_fft(a.md, (int64_t)N, p.subgrid_size, p.grid_size, g.planes,
                             static_cast<const float2 *>(g.dev), a.subgrids, a.taper, st));
        chk(launch_degridder(a, variant, p.nr_channels, st));
    }
    if (j.k1) chk(cudaEventRecord(j.k1, st));
    if (j.spec.op == IDG_JOB_DEGRID)
        chk(cudaMemcpyAsync(j.spec.vis_out, dp(L.vis), b_vis, cudaMemcpyDeviceToHost, st));
    if (j.c1) chk(cudaEventRecord(j.c1, st));
    chk(cudaEventRecord(j.done, st));
    if (g.last_op != j.spec.op) g.holders.clear();
    g.last_op = j.spec.op;
    g.holders.push_back(j.done);
    if (e != cudaSuccess) j.status = cuda_fail(e, "server job launch");
}

void idg_server::admit_locked() {
    // grids with a job left waiting in this scan: later jobs on them must not overtake it
    std::vector<int64_t> blocked;
    auto is_blocked = [&](int64_t g) { return std::find(blocked.begin(), blocked.end(), g) != blocked.end(); };
    for (auto it = queue.begin(); it != queue.end();) {
        int free_slot = -1;
        for (int s = 0; s < (int)slots.size(); ++s)
            if (!slots[s]) {
                free_slot = s;
                break;
            }
        if (free_slot < 0) return;
        Job &j = **it;
        // a gridding job must not change a grid while idg_server_grid_read copies it out
        const bool grid_being_read = j.spec.op == IDG_JOB_GRID && grids[j.spec.grid_id].readers > 0;
        if (is_blocked(j.spec.grid_id) || grid_being_read || in_use + j.footprint > (size_t)cfg.hbm_budget_bytes) {
            blocked.push_back(j.spec.grid_id);
            ++it; // a smaller job behind it, on another grid, may fit now
            continue;
        }
        cudaSetDevice(device);
        void *arena = nullptr;
        cudaError_t e = cudaMallocAsync(&arena, j.footprint, streams[free_slot]);
        if (e != cudaSuccess) {
            cudaGetLastError();
            blocked.push_back(j.spec.grid_id);
            ++it; // the pool cannot serve it right now; retry when memory frees up
            continue;
        }
        j.arena = arena;
        j.slot = free_slot;
        j.t_admit = Clock::now();
        slots[free_slot] = *it;
        in_use += j.footprint;
        peak_use = std::max(peak_use, in_use);
        cudaEventCreateWithFlags(&j.done, cudaEventDisableTiming);
        if (j.spec.op == IDG_JOB_GRID && cudaEventCreateWithFlags(&j.add_done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            j.add_done = nullptr; // the job's end event stands in for it
        }
        if (cudaEventCreate(&j.k0) != cudaSuccess || cudaEventCreate(&j.k1) != cudaSuccess) {
            cudaGetLastError();
            if (j.k0) cudaEventDestroy(j.k0);
            j.k0 = j.k1 = nullptr; // the job runs without its device interval
        }
        if (cudaEventCreate(&j.c0) != cudaSuccess || cudaEventCreate(&j.c1) != cudaSuccess) {
            cudaGetLastError();
            if (j.c0) cudaEventDestroy(j.c0);
            j.c0 = j.c1 = nullptr; // ... and without its stream interval
        }
        launch(j);
        it = queue.erase(it);
        cv_done.notify_all(); // a grid read may be waiting for this job's admission
    }
}

void idg_server::poll_locked() {
    for (int s = 0; s < (int)slots.size(); ++s) {
        auto &jp = slots[s];
        if (!jp) continue;
        // The slot's stream holds only this job's work (and earlier, finished
        // work): the job is over when the stream is idle.  Querying the stream
        // rather than the job's event also covers a launch that failed part way,
        // whose later copies and kernels may still be queued.
        cudaError_t q = cudaStreamQuery(streams[s]);
        if (q == cudaErrorNotReady) continue;
        Job &j = *jp;
        j.t_done = Clock::now();
        if (q != cudaSuccess && j.status == IDG_OK) j.status = cuda_fail(q, "server job");
        if (j.k0 && j.k1 && q == cudaSuccess && j.status == IDG_OK) {
            float t0 = 0, t1 = 0;
            if (cudaEventElapsedTime(&t0, epoch, j.k0) == cudaSuccess &&
                cudaEventElapsedTime(&t1, epoch, j.k1) == cudaSuccess) {
                j.dev_start_ms = t0;
                j.dev_end_ms = t1;
                // the rate estimate: only jobs that ran alone measure the full budget
                const double gpv = (double)j.nvis * j.spec.params.subgrid_size * j.spec.params.subgrid_size * 1e-9;
                if (j.share == 1 && gpv > 0.5 && t1 > t0) ms_per_gpv = 0.8 * ms_per_gpv + 0.2 * ((t1 - t0) / gpv);
            } else {
                cudaGetLastError();
            }
        }
        if (j.c0 && j.c1 && q == cudaSuccess && j.status == IDG_OK) {
            float t0 = 0, t1 = 0;
            if (cudaEventElapsedTime(&t0, epoch, j.c0) == cudaSuccess &&
                cudaEventElapsedTime(&t1, epoch, j.c1) == cudaSuccess) {
                j.work_start_ms = t0;
                j.work_end_ms = t1;
            } else {
                cudaGetLastError();
            }
        }
        if (j.k0) cudaEventDestroy(j.k0);
        if (j.k1) cudaEventDestroy(j.k1);
        if (j.c0) cudaEventDestroy(j.c0);
        if (j.c1) cudaEventDestroy(j.c1);
        j.k0 = j.k1 = j.c0 = j.c1 = nullptr;
        // plan entries the kernels rejected
        if (j.status == IDG_OK) {
            unsigned st = 0;
            const Layout L = job_layout(j.spec, j.spec.op == IDG_JOB_GRID ? &j.bins : nullptr);
            cudaMemcpy(&st, static_cast<char *>(j.arena) + L.words + 8, sizeof st, cudaMemcpyDeviceToHost);
            if (st) j.status = IDG_ERR_DEVICE_CHECK;
        }
        Grid &g = grids[j.spec.grid_id];
        g.holders.erase(std::remove(g.holders.begin(), g.holders.end(), j.done), g.holders.end());
        if (g.holders.empty()) g.last_op = -1;
        if (g.last_add && (g.last_add == j.add_done || g.last_add == j.done))
            g.last_add = nullptr; // finished: later adders need not wait for it
        if (j.add_done) {
            cudaEventDestroy(j.add_done);
            j.add_done = nullptr;
        }
        cudaFreeAsync(j.arena, streams[s]);
        cudaEventDestroy(j.done);
        j.done = nullptr;
        j.arena = nullptr;
        in_use -= j.footprint;
        j.finished = true;
        if (j.status == IDG_OK) {
            ++completed;
            total_vis += j.nvis;
            latencies.push_back(ms_between(j.t_submit, j.t_done));
            last_done = j.t_done;
        } else {
            ++failed;
        }
        jp.reset();
        cv_done.notify_all();
    }
}

void idg_server::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(mu);
    for (;;) {
        poll_locked();
        admit_locked();
        bool running = false;
        for (auto &s : slots)
            if (s) running = true;
        if (stop && !running && queue.empty()) break;
        // short sleep while kernels run; wake at once on new work
        cv_work.wait_for(lock, std::chrono::microseconds(running ? 100 : 2000));
    }
}

extern "C" {

IDG_API int idg_server_create(const idg_server_config *cfg, idg_server **out) {
    if (!cfg || !out) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->max_slots < 1 || cfg->max_slots > 64) return fail(IDG_ERR_INVALID_ARGUMENT, "max_slots %d", cfg->max_slots);
    if (cfg->hbm_budget_bytes < (1 << 20)) return fail(IDG_ERR_INVALID_ARGUMENT, "hbm budget too small");
    auto *srv = new idg_server;
    srv->cfg = *cfg;
    cudaGetDevice(&srv->device);
    srv->slots.resize(cfg->max_slots);
    srv->streams.resize(cfg->max_slots);
    // Job arenas come from the device's default stream-ordered pool.  Keep up
    // to the budget in it across synchronisations, so that a job's arena is
    // carved from memory a finished job returned rather than mapped anew
    // (the pool's default is to give unused memory back at every sync).
    {
        cudaMemPool_t pool = nullptr;
        if (cudaDeviceGetDefaultMemPool(&pool, srv->device) == cudaSuccess) {
            uint64_t keep = (uint64_t)cfg->hbm_budget_bytes, have = 0;
            if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &have) == cudaSuccess && have < keep)
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    for (auto &s : srv->streams) {
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            for (auto &t : srv->streams)
                if (t) cudaStreamDestroy(t);
            delete srv;
            return cuda_fail(e, "server stream");
        }
    }
    if (cudaEventCreate(&srv->epoch) != cudaSuccess || cudaEventRecord(srv->epoch, srv->streams[0]) != cudaSuccess ||
        cudaEventSynchronize(srv->epoch) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        if (srv->epoch) cudaEventDestroy(srv->epoch);
        for (auto &t : srv->streams) cudaStreamDestroy(t);
        delete srv;
        return cuda_fail(e, "server epoch event");
    }
    // keep freed job memory in the pool between jobs
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, srv->device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    srv->worker = std::thread([srv] { srv->run(); });
    *out = srv;
    return IDG_OK;
}

IDG_API int idg_server_destroy(idg_server *srv) {
    if (!srv) return IDG_OK;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    srv->worker.join();
    cudaSetDevice(srv->device);
    for (auto &g : srv->grids) cudaFree(g.second.dev);
    for (auto &s : srv->streams) cudaStreamDestroy(s);
    cudaEventDestroy(srv->epoch);
    delete srv;
    return IDG_OK;
}

IDG_API int idg_server_grid_create(idg_server *srv, int32_t grid_size, int32_t nr_w_planes, int64_t *grid_id) {
    if (!srv || !grid_id) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (grid_size < 1 || nr_w_planes < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "bad grid size");
    Grid g;
    g.size = grid_size;
    g.planes = nr_w_planes;
    g.bytes = (size_t)nr_w_planes * 4 * grid_size * grid_size * 8;
    cudaSetDevice(srv->device);
    IDG_CUDA(cudaMalloc(&g.dev, g.bytes));
    IDG_CUDA(cudaMemset(g.dev, 0, g.bytes));
    std::lock_guard<std::mutex> lock(srv->mu);
    *grid_id = srv->next_grid++;
    srv->grids[*grid_id] = g;
    return IDG_OK;
}

IDG_API int idg_server_grid_read(idg_server *srv, int64_t grid_id, void *host_out) {
    if (!srv || !host_out) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    IDG_CUDA(cudaSetDevice(srv->device));
    // The read covers every job on the grid submitted before it: first wait
    // until those have all been admitted.  The copy then runs on a stream of
    // its own.  Under the lock that stream is made to wait for every job now
    // holding the grid (the scheduler destroys a holder's event only under the
    // same lock), and the grid is marked as being read: until the copy ends,
    // the scheduler admits no gridding job on it and idg_server_grid_release
    // refuses it.
    cudaStream_t rs = nullptr;
    IDG_CUDA(cudaStreamCreateWithFlags(&rs, cudaStreamNonBlocking));
    void *dev = nullptr;
    size_t bytes = 0;
    {
        std::unique_lock<std::mutex> lock(srv->mu);
        const int64_t last_job = srv->next_job - 1;
        auto queued_before = [&] {
            for (auto &q : srv->queue)
                if (q->spec.grid_id == grid_id && q->id <= last_job) return true;
            return false;
        };
        if (!srv->cv_done.wait_for(lock, std::chrono::minutes(10), [&] { return !queued_before(); })) {
            cudaStreamDestroy(rs);
            return fail(IDG_ERR_TIMEOUT, "grid %lld: earlier jobs not admitted within 10 minutes", (long long)grid_id);
        }
        auto it = srv->grids.find(grid_id);
        if (it == srv->grids.end()) {
            cudaStreamDestroy(rs);
            return fail(IDG_ERR_NOT_FOUND, "unknown grid %lld", (long long)grid_id);
        }
        Grid &g = it->second;
        cudaError_t e = cudaSuccess;
        for (cudaEvent_t h : g.holders)
            if (e == cudaSuccess) e = cudaStreamWaitEvent(rs, h, 0);
        if (e != cudaSuccess) {
            cudaStreamDestroy(rs);
            return cuda_fail(e, "grid read: wait for the grid's jobs");
        }
        ++g.readers;
        dev = g.dev;
        bytes = g.bytes;
    }
    cudaError_t e = cudaMemcpyAsync(host_out, dev, bytes, cudaMemcpyDeviceToHost, rs);
    const cudaError_t e2 = cudaStreamSynchronize(rs);
    if (e == cudaSuccess) e = e2;
    cudaStreamDestroy(rs);
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        --srv->grids[grid_id].readers;
    }
    srv->cv_work.notify_all(); // gridding jobs held back by the read may start
    if (e != cudaSuccess) return cuda_fail(e, "grid read");
    return IDG_OK;
}

IDG_API int idg_server_grid_release(idg_server *srv, int64_t grid_id) {
    if (!srv) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->grids.find(grid_id);
    if (it == srv->grids.end()) return fail(IDG_ERR_NOT_FOUND, "unknown grid %lld", (long long)grid_id);
    if (!it->second.holders.empty()) return fail(IDG_ERR_REJECTED, "grid %lld has jobs in flight", (long long)grid_id);
    if (it->second.readers > 0) return fail(IDG_ERR_REJECTED, "grid %lld is being read", (long long)grid_id);
    for (auto &q : srv->queue)
        if (q->spec.grid_id == grid_id) return fail(IDG_ERR_REJECTED, "grid %lld has queued jobs", (long long)grid_id);
    cudaSetDevice(srv->device);
    cudaFree(it->second.dev);
    srv->grids.erase(it);
    return IDG_OK;
}

IDG_API int idg_server_submit(idg_server *srv, const idg_job *job, int64_t *job_id) {
    if (!srv || !job_id) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    auto j = std::make_shared<Job>();
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        if (int rc = validate_job(srv, job)) return rc;
    }
    j->spec = *job;
    const int64_t N = job->nr_subgrids;
    j->md.assign(job->metadata, job->metadata + N);
    if (job->ext) j->ext.assign(job->ext, job->ext + N);
    std::vector<int64_t> cost(N);
    for (int64_t s = 0; s < N; ++s) {
        const int nc = job->ext ? job->ext[s].channel_end - job->ext[s].channel_begin : job->params.nr_channels;
        cost[s] = (int64_t)job->metadata[s].nr_timesteps * nc;
        j->nvis += cost[s];
    }
    j->work.resize(N);
    std::iota(j->work.begin(), j->work.end(), 0);
    std::stable_sort(j->work.begin(), j->work.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    if (job->op == IDG_JOB_GRID)
        if (int rc = bin_tiles(&job->params, N, job->metadata, &j->bins)) return rc;
    j->footprint = job_layout(j->spec, job->op == IDG_JOB_GRID ? &j->bins : nullptr).total;
    std::lock_guard<std::mutex> lock(srv->mu);
    if (j->footprint > (size_t)srv->cfg.hbm_budget_bytes) {
        ++srv->rejected;
        return fail(IDG_ERR_REJECTED, "job needs %zu bytes of device memory, the budget is %lld", j->footprint,
                    (long long)srv->cfg.hbm_budget_bytes);
    }
    j->id = srv->next_job++;
    j->t_submit = Clock::now();
    if (!srv->have_first) {
        srv->first_submit = j->t_submit;
        srv->have_first = true;
    }
    srv->jobs[j->id] = j;
    srv->queue.push_back(j);
    *job_id = j->id;
    srv->cv_work.notify_all();
    return IDG_OK;
}

IDG_API int idg_server_wait(idg_server *srv, int64_t job_id, int64_t timeout_ms, idg_job_stats *stats) {
    if (!srv) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL server");
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return fail(IDG_ERR_NOT_FOUND, "unknown job %lld", (long long)job_id);
    std::shared_ptr<Job> j = it->second;
    const bool ok = srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                          [&] { return j->finished; });
    if (!ok) return fail(IDG_ERR_TIMEOUT, "job %lld not finished after %lld ms", (long long)job_id, (long long)timeout_ms);
    if (stats) {
        stats->queue_ms = ms_between(j->t_submit, j->t_admit);
        stats->run_ms = ms_between(j->t_admit, j->t_done);
        stats->latency_ms = ms_between(j->t_submit, j->t_done);
        stats->visibilities = j->nvis;
        stats->status = j->status;
        stats->device_start_ms = j->dev_start_ms;
        stats->device_end_ms = j->dev_end_ms;
        stats->stream_start_ms = j->work_start_ms;
        stats->stream_end_ms = j->work_end_ms;
    }
    srv->jobs.erase(job_id);
    if (j->status != IDG_OK) return fail(j->status, "job %lld failed", (long long)job_id);
    return IDG_OK;
}

IDG_API int idg_server_stats(idg_server *srv, idg_server_summary *out) {
    if (!srv || !out) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(srv->mu);
    memset(out, 0, sizeof *out);
    out->completed = srv->completed;
    out->rejected = srv->rejected;
    out->failed = srv->failed;
    out->queued = (int64_t)srv->queue.size();
    int running = 0;
    for (auto &s : srv->slots)
        if (s) ++running;
    out->running = running;
    out->hbm_in_use = (int64_t)srv->in_use;
    out->hbm_peak = (int64_t)srv->peak_use;
    std::vector<double> l = srv->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) { return l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->mean_ms = std::accumulate(l.begin(), l.end(), 0.0) / l.size();
        const double span_s = ms_between(srv->first_submit, srv->last_done) * 1e-3;
        out->mvis_per_s = span_s > 0 ? srv->total_vis / span_s / 1e6 : 0;
    }
    return IDG_OK;
}

} // extern "C"
