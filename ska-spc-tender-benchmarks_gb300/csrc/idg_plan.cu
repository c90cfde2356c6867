// idg_plan.cu -- device-resident execution plans and their CUDA graphs.
//
// A plan holds everything about a set of subgrids that does not change from
// one imaging cycle to the next: the metadata and channel sidecar on the
// device, a work list that orders the subgrids longest first (so that the
// persistent kernels finish uneven subgrids together), its own work counter
// and check word (so plans on different streams never share scheduler
// state), and the subgrid work space.  A plan can capture a whole cycle --
// zero the grid, gridder -> FFT -> adder, splitter -> FFT -> degridder -- into
// one CUDA graph and replay it with a single launch.  The plan's adder sums
// in a fixed order (tile bins made from the host metadata at creation,
// idg_tiles.cu), so a plan's grid is the same bit for bit on every run.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"
#include "idg_tiles.h"

struct idg_plan {
    idg_params params{};
    int variant = IDG_VARIANT_BATCHED;
    int device = 0;
    int64_t nr_subgrids = 0, nr_rows = 0;
    int max_ctas = 0;
    idg_metadata *d_md = nullptr;
    idg_subgrid_ext *d_ext = nullptr;
    int *d_work = nullptr;
    unsigned *d_words = nullptr; // [0] gridder counter, [1] degridder counter, [2] check word
    void *d_subgrids = nullptr;
    void *bins_mem = nullptr; // the adder's tile bins (and their own metadata copy)
    idg::TileBinsDev bins;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
};

// A captured cycle over several plans sharing one grid (idg_cycle_capture).
struct idg_cycle {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
};

namespace {

using namespace idg;

void plan_free(idg_plan *p) {
    if (!p) return;
    if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    for (void *q : {(void *)p->d_md, (void *)p->d_ext, (void *)p->d_work, (void *)p->d_words, p->d_subgrids, p->bins_mem})
        if (q) cudaFree(q);
    delete p;
}

KernelArgs plan_args(const idg_plan *p, const float *uvw, const float *k, const float *taper, const void *aterms,
                     void *vis, void *subgrids, bool degrid) {
    KernelArgs a{};
    const idg_params &q = p->params;
    a.G = q.grid_size;
    a.S = q.subgrid_size;
    a.C = q.nr_channels;
    a.nr_stations = q.nr_stations;
    a.nr_aterms = q.nr_aterms;
    a.nr_w_planes = q.nr_w_planes > 0 ? q.nr_w_planes : 1;
    a.image_size = q.image_size;
    a.w_step = q.w_step;
    a.flags = q.flags | IDG_FLAG_NO_TAPER; // the FFT applies the taper
    a.nr_subgrids = p->nr_subgrids;
    a.nr_rows = p->nr_rows;
    a.md = p->d_md;
    a.ext = p->d_ext;
    a.uvw = uvw;
    a.wavenumbers = k;
    a.taper = taper;
    a.aterms = reinterpret_cast<const float4 *>(aterms);
    a.vis = reinterpret_cast<float4 *>(vis);
    a.subgrids = reinterpret_cast<float2 *>(subgrids);
    a.work_list = p->d_work;
    a.work_counter = reinterpret_cast<int *>(p->d_words) + (degrid ? 1 : 0);
    a.status = p->d_words + 2;
    a.max_ctas = p->max_ctas;
    return a;
}

bool aligned16(const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; }

int check_data(const idg_plan *p, const float *uvw, const float *k, const void *vis, const float *taper,
               const void *aterms, const void *grid) {
    if (!p) return fail(IDG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!uvw || !k || !vis || !taper || !aterms || !grid) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (!aligned16(vis) || !aligned16(aterms) || !aligned16(grid))
        return fail(IDG_ERR_INVALID_ARGUMENT, "visibilities, aterms and grid must be 16-byte aligned");
    int dev = 0;
    IDG_CUDA(cudaGetDevice(&dev));
    if (dev != p->device) return fail(IDG_ERR_INVALID_ARGUMENT, "plan belongs to device %d, current is %d", p->device, dev);
    return IDG_OK;
}

int grid_step(idg_plan *p, const float *uvw, const float *k, const void *vis, const float *taper, const void *aterms,
              void *grid, cudaStream_t st) {
    const idg_params &q = p->params;
    if (p->variant == IDG_VARIANT_BATCHED) IDG_CUDA(cudaMemsetAsync(p->d_words, 0, sizeof(int), st));
    KernelArgs a = plan_args(p, uvw, k, taper, aterms, const_cast<void *>(vis), p->d_subgrids, false);
    cudaError_t e = launch_gridder(a, p->variant, q.nr_channels, st);
    if (e != cudaSuccess) return cuda_fail(e, "plan gridder");
    e = launch_subgrid_fft(reinterpret_cast<float2 *>(p->d_subgrids), p->nr_subgrids, q.subgrid_size, +1, taper, st);
    if (e != cudaSuccess) return cuda_fail(e, "plan subgrid fft");
    e = launch_binned_adder(p->bins, reinterpret_cast<const float2 *>(p->d_subgrids), reinterpret_cast<float2 *>(grid),
                            st);
    if (e != cudaSuccess) return cuda_fail(e, "plan adder");
    return IDG_OK;
}

int degrid_step(idg_plan *p, const float *uvw, const float *k, void *vis_out, const float *taper, const void *aterms,
                const void *grid, cudaStream_t st) {
    const idg_params &q = p->params;
    // splitter and backward subgrid FFT in one pass
    cudaError_t e = launch_split_fft(p->d_md, p->nr_subgrids, q.subgrid_size, q.grid_size,
                                     q.nr_w_planes > 0 ? q.nr_w_planes : 1, reinterpret_cast<const float2 *>(grid),
                                     reinterpret_cast<float2 *>(p->d_subgrids), taper, st);
    if (e != cudaSuccess) return cuda_fail(e, "plan split + subgrid fft");
    if (p->variant == IDG_VARIANT_BATCHED)
        IDG_CUDA(cudaMemsetAsync(reinterpret_cast<int *>(p->d_words) + 1, 0, sizeof(int), st));
    KernelArgs a = plan_args(p, uvw, k, taper, aterms, vis_out, p->d_subgrids, true);
    e = launch_degridder(a, p->variant, q.nr_channels, st);
    if (e != cudaSuccess) return cuda_fail(e, "plan degridder");
    return IDG_OK;
}

} // namespace

extern "C" {

IDG_API int idg_plan_create(const idg_params *params, int variant, int64_t nr_subgrids, const idg_metadata *metadata,
                            const idg_subgrid_ext *ext, int64_t nr_rows, idg_plan **plan) {
    if (!plan) return fail(IDG_ERR_INVALID_ARGUMENT, "plan output is NULL");
    *plan = nullptr;
    if (int rc = check_params(params, true)) return rc;
    if (variant != IDG_VARIANT_PLAIN && variant != IDG_VARIANT_BATCHED)
        return fail(IDG_ERR_INVALID_ARGUMENT, "unknown variant %d", variant);
    if (nr_subgrids < 1 || nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids %lld", (long long)nr_subgrids);
    if (!metadata) return fail(IDG_ERR_INVALID_ARGUMENT, "metadata is NULL");
    // validate on the host and order by cost (visibilities per subgrid), longest first
    const int bo1 = metadata[0].baseline_offset;
    std::vector<int64_t> cost(nr_subgrids);
    for (int64_t s = 0; s < nr_subgrids; ++s) {
        const idg_metadata &m = metadata[s];
        const int64_t r0 = (int64_t)(m.baseline_offset - bo1) + m.time_offset;
        int c0 = 0, c1 = params->nr_channels;
        if (ext) {
            c0 = ext[s].channel_begin;
            c1 = ext[s].channel_end;
        }
        if (r0 < 0 || m.nr_timesteps < 0 || r0 + m.nr_timesteps > nr_rows || m.station1 >= (uint32_t)params->nr_stations ||
            m.station2 >= (uint32_t)params->nr_stations || m.aterm_index < 0 || m.aterm_index >= params->nr_aterms ||
            c0 < 0 || c1 > params->nr_channels || c0 > c1)
            return fail(IDG_ERR_INVALID_ARGUMENT, "plan entry %lld is out of range", (long long)s);
        cost[s] = (int64_t)m.nr_timesteps * (c1 - c0);
    }
    std::vector<int> order(nr_subgrids);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });

    TileBinsHost bins;
    if (int rc = bin_tiles(params, nr_subgrids, metadata, &bins)) return rc;

    idg_plan *p = new idg_plan;
    p->params = *params;
    p->variant = variant;
    p->nr_subgrids = nr_subgrids;
    p->nr_rows = nr_rows;
    cudaGetDevice(&p->device);
    const int64_t S = params->subgrid_size;
    auto bail = [&](cudaError_t e, const char *what) {
        plan_free(p);
        return cuda_fail(e, what);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&p->d_md, sizeof(idg_metadata) * nr_subgrids)) != cudaSuccess) return bail(e, "plan metadata");
    if (ext && (e = cudaMalloc(&p->d_ext, sizeof(idg_subgrid_ext) * nr_subgrids)) != cudaSuccess)
        return bail(e, "plan sidecar");
    if ((e = cudaMalloc(&p->d_work, sizeof(int) * nr_subgrids)) != cudaSuccess) return bail(e, "plan work list");
    if ((e = cudaMalloc(&p->d_words, 256)) != cudaSuccess) return bail(e, "plan words");
    if ((e = cudaMalloc(&p->d_subgrids, (size_t)nr_subgrids * 4 * S * S * 8)) != cudaSuccess)
        return bail(e, "plan subgrid work space");
    if ((e = cudaMemcpy(p->d_md, metadata, sizeof(idg_metadata) * nr_subgrids, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(e, "plan metadata copy");
    if (ext && (e = cudaMemcpy(p->d_ext, ext, sizeof(idg_subgrid_ext) * nr_subgrids, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(e, "plan sidecar copy");
    if ((e = cudaMemcpy(p->d_work, order.data(), sizeof(int) * nr_subgrids, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(e, "plan work list copy");
    if ((e = cudaMemset(p->d_words, 0, 256)) != cudaSuccess) return bail(e, "plan words clear");
    if (int rc = upload_tile_bins(bins, nr_subgrids, metadata, &p->bins_mem, &p->bins)) {
        plan_free(p);
        return rc;
    }
    *plan = p;
    return IDG_OK;
}

IDG_API int idg_plan_destroy(idg_plan *plan) {
    plan_free(plan);
    return IDG_OK;
}

IDG_API int idg_plan_set_cta_limit(idg_plan *plan, int max_ctas) {
    if (!plan) return fail(IDG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (max_ctas < 0) return fail(IDG_ERR_INVALID_ARGUMENT, "max_ctas < 0");
    plan->max_ctas = max_ctas;
    return IDG_OK;
}

IDG_API int idg_plan_grid(idg_plan *plan, const float *uvw, const float *wavenumbers, const void *visibilities,
                          const float *spheroidal, const void *aterms, void *grid, void *stream) {
    if (int rc = check_data(plan, uvw, wavenumbers, visibilities, spheroidal, aterms, grid)) return rc;
    return grid_step(plan, uvw, wavenumbers, visibilities, spheroidal, aterms, grid, reinterpret_cast<cudaStream_t>(stream));
}

IDG_API int idg_plan_degrid(idg_plan *plan, const float *uvw, const float *wavenumbers, void *visibilities,
                            const float *spheroidal, const void *aterms, const void *grid, void *stream) {
    if (int rc = check_data(plan, uvw, wavenumbers, visibilities, spheroidal, aterms, grid)) return rc;
    return degrid_step(plan, uvw, wavenumbers, visibilities, spheroidal, aterms, grid,
                       reinterpret_cast<cudaStream_t>(stream));
}

IDG_API int idg_plan_capture_cycle(idg_plan *plan, const float *uvw, const float *wavenumbers,
                                   const void *visibilities_in, const float *spheroidal, const void *aterms, void *grid,
                                   void *visibilities_out) {
    if (int rc = check_data(plan, uvw, wavenumbers, visibilities_in, spheroidal, aterms, grid)) return rc;
    if (!visibilities_out || !aligned16(visibilities_out))
        return fail(IDG_ERR_INVALID_ARGUMENT, "visibilities_out must be a 16-byte aligned device pointer");
    if (plan->graph_exec) {
        cudaGraphExecDestroy(plan->graph_exec);
        plan->graph_exec = nullptr;
    }
    if (plan->graph) {
        cudaGraphDestroy(plan->graph);
        plan->graph = nullptr;
    }
    const idg_params &q = plan->params;
    const size_t b_grid = (size_t)(q.nr_w_planes > 0 ? q.nr_w_planes : 1) * 4 * q.grid_size * q.grid_size * 8;
    cudaStream_t st = nullptr;
    IDG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    int rc = IDG_OK;
    if (e == cudaSuccess) {
        e = cudaMemsetAsync(grid, 0, b_grid, st);
        if (e == cudaSuccess) {
            rc = grid_step(plan, uvw, wavenumbers, visibilities_in, spheroidal, aterms, grid, st);
            if (!rc) rc = degrid_step(plan, uvw, wavenumbers, visibilities_out, spheroidal, aterms, grid, st);
        }
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(st, &g);
        if (e == cudaSuccess) e = e2;
        plan->graph = g;
    }
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "graph capture of the imaging cycle");
    IDG_CUDA(cudaGraphInstantiate(&plan->graph_exec, plan->graph, 0));
    return IDG_OK;
}

IDG_API int idg_plan_launch_cycle(idg_plan *plan, void *stream) {
    if (!plan || !plan->graph_exec) return fail(IDG_ERR_INVALID_ARGUMENT, "plan has no captured cycle");
    IDG_CUDA(cudaGraphLaunch(plan->graph_exec, reinterpret_cast<cudaStream_t>(stream)));
    return IDG_OK;
}

IDG_API int idg_cycle_capture(int nr_plans, idg_plan *const *plans, const float *const *uvw,
                              const float *const *wavenumbers, const void *const *visibilities_in,
                              const float *const *spheroidal, const void *const *aterms, void *grid,
                              void *const *visibilities_out, idg_cycle **cycle) {
    if (!cycle) return fail(IDG_ERR_INVALID_ARGUMENT, "cycle output is NULL");
    *cycle = nullptr;
    if (nr_plans < 1 || !plans || !uvw || !wavenumbers || !visibilities_in || !spheroidal || !aterms ||
        !visibilities_out)
        return fail(IDG_ERR_INVALID_ARGUMENT, "nr_plans %d or a NULL array", nr_plans);
    const idg_params &q0 = plans[0] ? plans[0]->params : idg_params{};
    for (int i = 0; i < nr_plans; ++i) {
        idg_plan *p = plans[i];
        if (!p) return fail(IDG_ERR_INVALID_ARGUMENT, "plan %d is NULL", i);
        if (p->params.grid_size != q0.grid_size || p->params.nr_w_planes != q0.nr_w_planes)
            return fail(IDG_ERR_INVALID_ARGUMENT, "plan %d: grid %d x %d planes differs from plan 0 (%d x %d)", i,
                        p->params.grid_size, p->params.nr_w_planes, q0.grid_size, q0.nr_w_planes);
        if (int rc = check_data(p, uvw[i], wavenumbers[i], visibilities_in[i], spheroidal[i], aterms[i], grid))
            return rc;
        if (!visibilities_out[i] || !aligned16(visibilities_out[i]))
            return fail(IDG_ERR_INVALID_ARGUMENT, "visibilities_out[%d] must be a 16-byte aligned device pointer", i);
    }
    auto *c = new idg_cycle();
    const size_t b_grid = (size_t)(q0.nr_w_planes > 0 ? q0.nr_w_planes : 1) * 4 * q0.grid_size * q0.grid_size * 8;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "stream for the cycle capture");
    }
    int rc = IDG_OK;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = cudaMemsetAsync(grid, 0, b_grid, st);
        for (int i = 0; e == cudaSuccess && !rc && i < nr_plans; ++i)
            rc = grid_step(plans[i], uvw[i], wavenumbers[i], visibilities_in[i], spheroidal[i], aterms[i], grid, st);
        for (int i = 0; e == cudaSuccess && !rc && i < nr_plans; ++i)
            rc = degrid_step(plans[i], uvw[i], wavenumbers[i], visibilities_out[i], spheroidal[i], aterms[i], grid, st);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(st, &g);
        if (e == cudaSuccess) e = e2;
        c->graph = g;
    }
    cudaStreamDestroy(st);
    if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&c->graph_exec, c->graph, 0);
    if (rc || e != cudaSuccess) {
        if (c->graph) cudaGraphDestroy(c->graph);
        delete c;
        return rc ? rc : cuda_fail(e, "graph capture of the multi-plan cycle");
    }
    *cycle = c;
    return IDG_OK;
}

IDG_API int idg_cycle_launch(idg_cycle *cycle, void *stream) {
    if (!cycle || !cycle->graph_exec) return fail(IDG_ERR_INVALID_ARGUMENT, "cycle is NULL or empty");
    IDG_CUDA(cudaGraphLaunch(cycle->graph_exec, reinterpret_cast<cudaStream_t>(stream)));
    return IDG_OK;
}

IDG_API int idg_cycle_destroy(idg_cycle *cycle) {
    if (!cycle) return IDG_OK;
    if (cycle->graph_exec) cudaGraphExecDestroy(cycle->graph_exec);
    if (cycle->graph) cudaGraphDestroy(cycle->graph);
    delete cycle;
    return IDG_OK;
}

IDG_API int idg_plan_status(idg_plan *plan, void *stream, uint32_t *status, int clear) {
    if (!plan || !status) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    IDG_CUDA(cudaStreamSynchronize(st));
    unsigned v = 0;
    IDG_CUDA(cudaMemcpy(&v, plan->d_words + 2, sizeof v, cudaMemcpyDeviceToHost));
    if (clear) IDG_CUDA(cudaMemset(plan->d_words + 2, 0, sizeof(unsigned)));
    *status = v;
    return IDG_OK;
}

} // extern "C"
