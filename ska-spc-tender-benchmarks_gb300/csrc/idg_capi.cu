// idg_capi.cu -- the extern "C" boundary (include/idg_gb300.h).
//
// Validates every call on the host, turns it into idg::KernelArgs and
// launches the kernels on the caller's stream.  The drop-in launchers
// (idg_gridding_launch / idg_degridding_launch) reproduce the reference's
// GPU launchers (gridding/src/gridding_benchmark.cu:248-361,
// gridding/src/degridding_benchmark.cu:205-318): allocate, copy in
// `niterations` times, run `niterations` times, copy out, report
// benchmark_result in microseconds and bytes per microsecond.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"

namespace idg {

int reference_dataset(int64_t grid_size, int64_t S, int64_t nstations, int64_t C, int64_t ntimeslots, int64_t T,
                      float image_size, float *uvw, float *frequencies, float *wavenumbers, void *visibilities,
                      uint32_t *baselines, float *spheroidal, void *aterms, idg_metadata *metadata);

namespace {
thread_local std::string g_last_error;
std::mutex g_words_mutex;
std::vector<DeviceWords> g_words;

// Launch shapes of the batched kernels per (device, subgrid size), set by the
// autotuner or by idg_set_batched_shapes().  Until then, the shapes measured
// fastest on GB300: the mirror-quad gridder with 64 threads x 4 quads (shape
// 22; 24 with 512-visibility tiles for S = 32) where 64 threads cover whole
// quad columns (S/2 divides 64), else the Gauss pixel-pair shapes that make
// whole passes for S = 24 (11) and 48 (12); the mirror-quad degridder with
// kappa from shared memory, in column form (shape 32; 34 with its runs of
// four quads for S = 32) or row by row (shape 31).
std::mutex g_shape_mutex;
std::map<std::pair<int, int>, std::pair<int, int>> g_shapes;

int current_device() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

// Degridder: the column form (32) where each lane's quads run down a column
// for at least four steps (S a multiple of 8, S >= 32), else the row form (31).
std::pair<int, int> default_shapes(int S) {
    const int g = S == 32 ? 24 : (S >= 2 && 64 % (S / 2) == 0) ? 22 : S == 24 ? 11 : S == 48 ? 12 : 13;
    const int d = S == 32 ? 34 : (S >= 32 && S % 8 == 0) ? 32 : 31;
    return {g < gridder_fast_shapes() ? g : 0, d < degridder_fast_shapes() ? d : 0};
}

std::pair<int, int> &shapes_of(int S) {
    auto it = g_shapes.find({current_device(), S});
    if (it == g_shapes.end()) it = g_shapes.emplace(std::make_pair(current_device(), S), default_shapes(S)).first;
    return it->second;
}
} // namespace

int batched_gridder_shape(int S) {
    std::lock_guard<std::mutex> lock(g_shape_mutex);
    return shapes_of(S).first;
}
int batched_degridder_shape(int S) {
    std::lock_guard<std::mutex> lock(g_shape_mutex);
    return shapes_of(S).second;
}
void set_batched_gridder_shape(int S, int shape) {
    std::lock_guard<std::mutex> lock(g_shape_mutex);
    shapes_of(S).first = shape;
}
void set_batched_degridder_shape(int S, int shape) {
    std::lock_guard<std::mutex> lock(g_shape_mutex);
    shapes_of(S).second = shape;
}

int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? IDG_ERR_OUT_OF_MEMORY : IDG_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

int device_words(DeviceWords *out) {
    int dev = 0;
    IDG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_words_mutex);
    if ((int)g_words.size() <= dev) g_words.resize(dev + 1);
    if (!g_words[dev].status) {
        void *p = nullptr;
        IDG_CUDA(cudaMalloc(&p, 256));
        IDG_CUDA(cudaMemset(p, 0, 256));
        g_words[dev].status = static_cast<unsigned *>(p);
        g_words[dev].counter = reinterpret_cast<int *>(static_cast<char *>(p) + 128);
    }
    *out = g_words[dev];
    return IDG_OK;
}

int check_params(const idg_params *p, bool need_fft_size) {
    if (!p) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    if (p->subgrid_size < 2 || p->subgrid_size > 64 || (p->subgrid_size & 1))
        return fail(IDG_ERR_UNSUPPORTED, "subgrid_size %d: must be even and in [2, 64]", p->subgrid_size);
    if (need_fft_size && !fft_size_supported(p->subgrid_size))
        return fail(IDG_ERR_UNSUPPORTED, "subgrid_size %d: the subgrid FFT supports 8, 16, 24, 32, 48, 64",
                    p->subgrid_size);
    if (p->grid_size < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "grid_size %d < 1", p->grid_size);
    if (p->nr_channels < 1 || p->nr_channels > 1024)
        return fail(IDG_ERR_UNSUPPORTED, "nr_channels %d: must be in [1, 1024]", p->nr_channels);
    if (p->nr_stations < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_stations %d < 1", p->nr_stations);
    if (p->nr_aterms < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_aterms %d < 1", p->nr_aterms);
    if (!(p->image_size > 0.f) || !(p->image_size < 2.f))
        return fail(IDG_ERR_INVALID_ARGUMENT, "image_size %g: must be in (0, 2) radians", p->image_size);
    return IDG_OK;
}

namespace {

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

KernelArgs make_args(const idg_params *p, int64_t nr_subgrids, const idg_metadata *md, const idg_subgrid_ext *ext,
                     int64_t nr_rows, const float *uvw, const float *k, const float *taper, const void *aterms,
                     void *vis, void *subgrids) {
    KernelArgs a{};
    a.G = p->grid_size;
    a.S = p->subgrid_size;
    a.C = p->nr_channels;
    a.nr_stations = p->nr_stations;
    a.nr_aterms = p->nr_aterms;
    a.nr_w_planes = p->nr_w_planes > 0 ? p->nr_w_planes : 1;
    a.image_size = p->image_size;
    a.w_step = p->w_step;
    a.flags = p->flags;
    a.nr_subgrids = nr_subgrids;
    a.nr_rows = nr_rows;
    a.md = md;
    a.ext = ext;
    a.uvw = uvw;
    a.wavenumbers = k;
    a.taper = taper;
    a.aterms = reinterpret_cast<const float4 *>(aterms);
    a.vis = reinterpret_cast<float4 *>(vis);
    a.subgrids = reinterpret_cast<float2 *>(subgrids);
    return a;
}

int run_kernel(bool gridding, const idg_params *params, int variant, int64_t nr_subgrids, const idg_metadata *md,
               const idg_subgrid_ext *ext, int64_t nr_rows, const float *uvw, const float *k, void *vis,
               const float *taper, const void *aterms, void *subgrids, void *stream) {
    if (int rc = check_params(params)) return rc;
    if (variant != IDG_VARIANT_PLAIN && variant != IDG_VARIANT_BATCHED)
        return fail(IDG_ERR_INVALID_ARGUMENT, "unknown variant %d", variant);
    if (nr_subgrids < 0 || nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids %lld", (long long)nr_subgrids);
    if (nr_subgrids == 0) return IDG_OK;
    if (nr_rows < 0) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_rows %lld < 0", (long long)nr_rows);
    if (!md || !uvw || !k || !vis || !aterms || !subgrids)
        return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (!taper && !(params->flags & IDG_FLAG_NO_TAPER))
        return fail(IDG_ERR_INVALID_ARGUMENT, "spheroidal is NULL and IDG_FLAG_NO_TAPER is not set");
    if (!aligned16(vis) || !aligned16(aterms) || !aligned16(subgrids))
        return fail(IDG_ERR_INVALID_ARGUMENT, "visibilities, aterms and subgrids must be 16-byte aligned");
    KernelArgs a = make_args(params, nr_subgrids, md, ext, nr_rows, uvw, k, taper, aterms, vis, subgrids);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    DeviceWords w;
    if (int rc = device_words(&w)) return rc;
    a.status = w.status;
    if (variant == IDG_VARIANT_BATCHED) {
        IDG_CUDA(cudaMemsetAsync(w.counter, 0, sizeof(int), st));
        a.work_counter = w.counter;
    }
    cudaError_t e = gridding ? launch_gridder(a, variant, params->nr_channels, st)
                             : launch_degridder(a, variant, params->nr_channels, st);
    if (e != cudaSuccess) return cuda_fail(e, gridding ? "gridder launch" : "degridder launch");
    return IDG_OK;
}

} // namespace
} // namespace idg

using namespace idg;

extern "C" {

IDG_API int idg_abi_version(void) { return IDG_ABI_VERSION; }

IDG_API const char *idg_last_error(void) { return g_last_error.c_str(); }

IDG_API int idg_device_status(void *stream, uint32_t *status, int clear) {
    if (!status) return fail(IDG_ERR_INVALID_ARGUMENT, "status is NULL");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    DeviceWords w;
    if (int rc = device_words(&w)) return rc;
    unsigned v = 0;
    IDG_CUDA(cudaStreamSynchronize(st));
    IDG_CUDA(cudaMemcpy(&v, w.status, sizeof v, cudaMemcpyDeviceToHost));
    if (clear) IDG_CUDA(cudaMemset(w.status, 0, sizeof(unsigned)));
    *status = v;
    return IDG_OK;
}

IDG_API int idg_gridder(const idg_params *params, int variant, int64_t nr_subgrids, const idg_metadata *metadata,
                        const idg_subgrid_ext *ext, int64_t nr_rows, const float *uvw, const float *wavenumbers,
                        const void *visibilities, const float *spheroidal, const void *aterms, void *subgrids,
                        void *stream) {
    return run_kernel(true, params, variant, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers,
                      const_cast<void *>(visibilities), spheroidal, aterms, subgrids, stream);
}

IDG_API int idg_degridder(const idg_params *params, int variant, int64_t nr_subgrids, const idg_metadata *metadata,
                          const idg_subgrid_ext *ext, int64_t nr_rows, const float *uvw, const float *wavenumbers,
                          void *visibilities, const float *spheroidal, const void *aterms, const void *subgrids,
                          void *stream) {
    return run_kernel(false, params, variant, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers, visibilities,
                      spheroidal, aterms, const_cast<void *>(subgrids), stream);
}

IDG_API int idg_subgrid_fft(const idg_params *params, int64_t nr_subgrids, int direction, const float *taper,
                            void *subgrids, void *stream) {
    if (!params) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    if (!fft_size_supported(params->subgrid_size))
        return fail(IDG_ERR_UNSUPPORTED, "subgrid_size %d: the subgrid FFT supports 8, 16, 24, 32, 48, 64",
                    params->subgrid_size);
    if (direction != 1 && direction != -1) return fail(IDG_ERR_INVALID_ARGUMENT, "direction %d: must be +1 or -1", direction);
    if (nr_subgrids < 0 || nr_subgrids * 4 / 1 > (int64_t)INT32_MAX * 64)
        return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids %lld", (long long)nr_subgrids);
    if (nr_subgrids == 0) return IDG_OK;
    if (!subgrids) return fail(IDG_ERR_INVALID_ARGUMENT, "subgrids is NULL");
    cudaError_t e = launch_subgrid_fft(reinterpret_cast<float2 *>(subgrids), nr_subgrids, params->subgrid_size,
                                       direction, taper, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "subgrid fft launch");
    return IDG_OK;
}

IDG_API int idg_adder(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                      const void *subgrids, void *grid, void *stream) {
    if (!params) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    if (params->subgrid_size < 1 || params->grid_size < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "bad sizes");
    if (nr_subgrids < 0 || nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids");
    if (nr_subgrids == 0) return IDG_OK;
    if (!metadata || !subgrids || !grid) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (!aligned16(subgrids) || !aligned16(grid)) return fail(IDG_ERR_INVALID_ARGUMENT, "subgrids/grid must be 16-byte aligned");
    cudaError_t e = launch_adder(metadata, nr_subgrids, params->subgrid_size, params->grid_size,
                                 params->nr_w_planes > 0 ? params->nr_w_planes : 1,
                                 reinterpret_cast<const float2 *>(subgrids), reinterpret_cast<float2 *>(grid),
                                 reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "adder launch");
    return IDG_OK;
}

IDG_API int idg_splitter(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                         const void *grid, void *subgrids, void *stream) {
    if (!params) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    if (params->subgrid_size < 1 || params->grid_size < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "bad sizes");
    if (nr_subgrids < 0 || nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids");
    if (nr_subgrids == 0) return IDG_OK;
    if (!metadata || !subgrids || !grid) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    cudaError_t e = launch_splitter(metadata, nr_subgrids, params->subgrid_size, params->grid_size,
                                    params->nr_w_planes > 0 ? params->nr_w_planes : 1,
                                    reinterpret_cast<const float2 *>(grid), reinterpret_cast<float2 *>(subgrids),
                                    reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "splitter launch");
    return IDG_OK;
}

IDG_API int idg_split_subgrid_fft(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                                  const void *grid, const float *spheroidal, void *subgrids, void *stream) {
    if (!params) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    if (!fft_size_supported(params->subgrid_size))
        return fail(IDG_ERR_UNSUPPORTED, "subgrid_size %d: the subgrid FFT supports 8, 16, 24, 32, 48, 64",
                    params->subgrid_size);
    if (params->grid_size < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "bad sizes");
    if (nr_subgrids < 0 || nr_subgrids > INT32_MAX) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids");
    if (nr_subgrids == 0) return IDG_OK;
    if (!metadata || !subgrids || !grid) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (!aligned16(subgrids)) return fail(IDG_ERR_INVALID_ARGUMENT, "subgrids must be 16-byte aligned");
    cudaError_t e = launch_split_fft(metadata, nr_subgrids, params->subgrid_size, params->grid_size,
                                     params->nr_w_planes > 0 ? params->nr_w_planes : 1,
                                     reinterpret_cast<const float2 *>(grid), reinterpret_cast<float2 *>(subgrids),
                                     spheroidal, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "split + subgrid fft launch");
    return IDG_OK;
}

IDG_API int idg_grid_fft(const idg_params *params, void *grid, int direction, const float *correction,
                         void *stream) {
    if (!params) return fail(IDG_ERR_INVALID_ARGUMENT, "params is NULL");
    const int G = params->grid_size, W = params->nr_w_planes > 0 ? params->nr_w_planes : 1;
    if (!grid_fft_size_supported(G))
        return fail(IDG_ERR_UNSUPPORTED, "grid size %d: the grid FFT takes powers of two from 64 to 8192", G);
    if (direction != 1 && direction != -1) return fail(IDG_ERR_INVALID_ARGUMENT, "direction must be +1 or -1");
    if (!grid || !aligned16(grid)) return fail(IDG_ERR_INVALID_ARGUMENT, "grid must be a 16-byte aligned device pointer");
    DeviceWords w;
    if (int rc = device_words(&w)) return rc;
    cudaError_t e = launch_grid_fft(reinterpret_cast<float2 *>(grid), G, 4 * W, direction, correction, w.status,
                                    (params->flags & IDG_FLAG_TEST_LOST_COPY) != 0,
                                    reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "grid FFT");
    return IDG_OK;
}

// ---------------------------------------------------------------------------
// Drop-in launchers
// ---------------------------------------------------------------------------
namespace {

struct DeviceBuffers {
    std::vector<void *> ptrs;
    ~DeviceBuffers() {
        for (void *p : ptrs) cudaFree(p);
    }
    int alloc(void **out, size_t bytes) {
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(out, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        ptrs.push_back(*out);
        return IDG_OK;
    }
};

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    int create() {
        IDG_CUDA(cudaEventCreate(&a));
        IDG_CUDA(cudaEventCreate(&b));
        return IDG_OK;
    }
    int elapsed_ms(float *ms) {
        IDG_CUDA(cudaEventSynchronize(b));
        IDG_CUDA(cudaEventElapsedTime(ms, a, b));
        return IDG_OK;
    }
};

int check_launch_config(const idg_launch_config *c, idg_params *p, int64_t *nsg, int64_t *nrows) {
    if (!c) return fail(IDG_ERR_INVALID_ARGUMENT, "config is NULL");
    if (c->niterations < 1) return fail(IDG_ERR_INVALID_ARGUMENT, "niterations %lld < 1", (long long)c->niterations);
    if (c->nstations < 2) return fail(IDG_ERR_INVALID_ARGUMENT, "nstations %lld < 2", (long long)c->nstations);
    if (c->ntimeslots < 1 || c->ntimesteps_per_subgrid < 1)
        return fail(IDG_ERR_INVALID_ARGUMENT, "ntimeslots and ntimesteps_per_subgrid must be >= 1");
    memset(p, 0, sizeof *p);
    p->grid_size = (int32_t)c->grid_size;
    p->subgrid_size = (int32_t)c->subgrid_size;
    p->nr_channels = (int32_t)c->nchannels;
    p->nr_stations = (int32_t)c->nstations;
    p->nr_aterms = (int32_t)c->ntimeslots;
    p->nr_w_planes = 1;
    p->image_size = c->image_size > 0.f ? c->image_size : 0.1F;
    p->w_step = c->w_step;
    p->flags = c->flags;
    if (int rc = check_params(p)) return rc;
    *nsg = c->nstations * (c->nstations - 1) / 2 * c->ntimeslots;
    *nrows = *nsg * c->ntimesteps_per_subgrid;
    return IDG_OK;
}

int host_launch(bool gridding, const idg_launch_config *config, const float *uvw, void *visibilities,
                const void *aterms, const float *wavenumbers, const float *spheroidal, void *subgrids,
                const idg_metadata *metadata, idg_benchmark_result *result) {
    idg_params p;
    int64_t nsg = 0, nrows = 0;
    if (int rc = check_launch_config(config, &p, &nsg, &nrows)) return rc;
    if (!uvw || !visibilities || !aterms || !wavenumbers || !spheroidal || !subgrids || !metadata)
        return fail(IDG_ERR_INVALID_ARGUMENT, "NULL host array");
    const int64_t S = p.subgrid_size, C = p.nr_channels;
    const size_t b_uvw = (size_t)nrows * 12, b_k = (size_t)C * 4, b_vis = (size_t)nrows * C * 32,
                 b_sph = (size_t)S * S * 4, b_at = (size_t)p.nr_aterms * p.nr_stations * S * S * 32,
                 b_md = (size_t)nsg * sizeof(idg_metadata), b_sub = (size_t)nsg * 4 * S * S * 8;
    DeviceBuffers buf;
    void *d_uvw, *d_k, *d_vis, *d_sph, *d_at, *d_md, *d_sub;
    if (int rc = buf.alloc(&d_uvw, b_uvw)) return rc;
    if (int rc = buf.alloc(&d_k, b_k)) return rc;
    if (int rc = buf.alloc(&d_vis, b_vis)) return rc;
    if (int rc = buf.alloc(&d_sph, b_sph)) return rc;
    if (int rc = buf.alloc(&d_at, b_at)) return rc;
    if (int rc = buf.alloc(&d_md, b_md)) return rc;
    if (int rc = buf.alloc(&d_sub, b_sub)) return rc;
    EventPair in, comp, out;
    if (int rc = in.create()) return rc;
    if (int rc = comp.create()) return rc;
    if (int rc = out.create()) return rc;

    const int64_t iters = config->niterations;
    size_t total_in = b_uvw + b_k + b_sph + b_at + b_md + (gridding ? b_vis : b_sub);
    IDG_CUDA(cudaEventRecord(in.a));
    for (int64_t i = 0; i < iters; ++i) {
        IDG_CUDA(cudaMemcpy(d_uvw, uvw, b_uvw, cudaMemcpyHostToDevice));
        IDG_CUDA(cudaMemcpy(d_k, wavenumbers, b_k, cudaMemcpyHostToDevice));
        if (gridding)
            IDG_CUDA(cudaMemcpy(d_vis, visibilities, b_vis, cudaMemcpyHostToDevice));
        else
            IDG_CUDA(cudaMemcpy(d_sub, subgrids, b_sub, cudaMemcpyHostToDevice));
        IDG_CUDA(cudaMemcpy(d_sph, spheroidal, b_sph, cudaMemcpyHostToDevice));
        IDG_CUDA(cudaMemcpy(d_at, aterms, b_at, cudaMemcpyHostToDevice));
        IDG_CUDA(cudaMemcpy(d_md, metadata, b_md, cudaMemcpyHostToDevice));
    }
    IDG_CUDA(cudaEventRecord(in.b));
    float in_ms = 0;
    if (int rc = in.elapsed_ms(&in_ms)) return rc;

    if (!gridding) IDG_CUDA(cudaMemset(d_vis, 0, b_vis));
    DeviceWords w;
    if (int rc = device_words(&w)) return rc;
    IDG_CUDA(cudaMemset(w.status, 0, sizeof(unsigned)));
    IDG_CUDA(cudaEventRecord(comp.a));
    for (int64_t i = 0; i < iters; ++i) {
        int rc = gridding ? idg_gridder(&p, config->variant, nsg, (const idg_metadata *)d_md, nullptr, nrows,
                                        (const float *)d_uvw, (const float *)d_k, d_vis, (const float *)d_sph, d_at,
                                        d_sub, nullptr)
                          : idg_degridder(&p, config->variant, nsg, (const idg_metadata *)d_md, nullptr, nrows,
                                          (const float *)d_uvw, (const float *)d_k, d_vis, (const float *)d_sph, d_at,
                                          d_sub, nullptr);
        if (rc) return rc;
    }
    IDG_CUDA(cudaEventRecord(comp.b));
    float comp_ms = 0;
    if (int rc = comp.elapsed_ms(&comp_ms)) return rc;
    unsigned status = 0;
    IDG_CUDA(cudaMemcpy(&status, w.status, sizeof status, cudaMemcpyDeviceToHost));
    if (status) return fail(IDG_ERR_DEVICE_CHECK, "a kernel rejected plan entries (status 0x%x)", status);

    const size_t total_out = gridding ? b_sub : b_vis;
    IDG_CUDA(cudaEventRecord(out.a));
    for (int64_t i = 0; i < iters; ++i) {
        if (gridding)
            IDG_CUDA(cudaMemcpy(subgrids, d_sub, b_sub, cudaMemcpyDeviceToHost));
        else
            IDG_CUDA(cudaMemcpy(visibilities, d_vis, b_vis, cudaMemcpyDeviceToHost));
    }
    IDG_CUDA(cudaEventRecord(out.b));
    float out_ms = 0;
    if (int rc = out.elapsed_ms(&out_ms)) return rc;

    if (result) {
        result->in_transfer_time = in_ms * 1000.0 / (double)iters;
        result->out_transfer_time = out_ms * 1000.0 / (double)iters;
        result->in_bandwidth = (double)total_in / (1000.0 * in_ms);
        result->out_bandwidth = (double)total_out / (1000.0 * out_ms);
        result->compute_time = comp_ms * 1000.0 / (double)iters;
    }
    return IDG_OK;
}

} // namespace

IDG_API int idg_gridding_launch(const idg_launch_config *config, const float *uvw, const void *visibilities,
                                const uint32_t *baselines, const void *aterms, const float *frequencies,
                                const float *wavenumbers, const float *spheroidal, void *subgrids,
                                const idg_metadata *metadata, idg_benchmark_result *result) {
    (void)baselines;
    (void)frequencies;
    return host_launch(true, config, uvw, const_cast<void *>(visibilities), aterms, wavenumbers, spheroidal, subgrids,
                       metadata, result);
}

IDG_API int idg_degridding_launch(const idg_launch_config *config, const float *uvw, void *visibilities,
                                  const uint32_t *baselines, const void *aterms, const float *frequencies,
                                  const float *wavenumbers, const float *spheroidal, const void *subgrids,
                                  const idg_metadata *metadata, idg_benchmark_result *result) {
    (void)baselines;
    (void)frequencies;
    return host_launch(false, config, uvw, visibilities, aterms, wavenumbers, spheroidal, const_cast<void *>(subgrids),
                       metadata, result);
}

IDG_API int idg_reference_dataset(int64_t grid_size, int64_t subgrid_size, int64_t nstations, int64_t nchannels,
                                  int64_t ntimeslots, int64_t ntimesteps_per_subgrid, float image_size, float *uvw,
                                  float *frequencies, float *wavenumbers, void *visibilities, uint32_t *baselines,
                                  float *spheroidal, void *aterms, idg_metadata *metadata) {
    if (grid_size < 1 || subgrid_size < 1 || nstations < 2 || nchannels < 1 || ntimeslots < 1 ||
        ntimesteps_per_subgrid < 1)
        return fail(IDG_ERR_INVALID_ARGUMENT, "bad reference dataset sizes");
    if (!uvw || !wavenumbers || !visibilities || !spheroidal || !aterms || !metadata)
        return fail(IDG_ERR_INVALID_ARGUMENT, "NULL host array");
    return reference_dataset(grid_size, subgrid_size, nstations, nchannels, ntimeslots, ntimesteps_per_subgrid,
                             image_size, uvw, frequencies, wavenumbers, visibilities, baselines, spheroidal, aterms,
                             metadata);
}

IDG_API int idg_batched_shapes(int *gridder_shapes, int *degridder_shapes) {
    if (!gridder_shapes || !degridder_shapes) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL output");
    *gridder_shapes = gridder_fast_shapes();
    *degridder_shapes = degridder_fast_shapes();
    return IDG_OK;
}

IDG_API int idg_set_batched_shapes(int subgrid_size, int gridder_shape, int degridder_shape) {
    if (gridder_shape < 0 || gridder_shape >= gridder_fast_shapes() || degridder_shape < 0 ||
        degridder_shape >= degridder_fast_shapes())
        return fail(IDG_ERR_INVALID_ARGUMENT, "shape out of range (gridder %d of %d, degridder %d of %d)", gridder_shape,
                    gridder_fast_shapes(), degridder_shape, degridder_fast_shapes());
    set_batched_gridder_shape(subgrid_size, gridder_shape);
    set_batched_degridder_shape(subgrid_size, degridder_shape);
    return IDG_OK;
}

IDG_API int idg_get_batched_shapes(int subgrid_size, int *gridder_shape, int *degridder_shape) {
    if (!gridder_shape || !degridder_shape) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL output");
    *gridder_shape = batched_gridder_shape(subgrid_size);
    *degridder_shape = batched_degridder_shape(subgrid_size);
    return IDG_OK;
}

namespace {
constexpr double kKeepMargin = 1.01;
}

IDG_API int idg_autotune(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                         const idg_subgrid_ext *ext, int64_t nr_rows, const float *uvw, const float *wavenumbers,
                         const void *visibilities, const float *spheroidal, const void *aterms, void *subgrids,
                         void *visibilities_out, void *stream, int repeats, double *gridder_ms, double *degridder_ms,
                         int *best_gridder, int *best_degridder) {
    if (!gridder_ms || !degridder_ms || !best_gridder || !best_degridder || !visibilities_out)
        return fail(IDG_ERR_INVALID_ARGUMENT, "NULL output");
    if (repeats < 1) repeats = 1;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    EventPair ev;
    if (int rc = ev.create()) return rc;
    const int S = params ? params->subgrid_size : 0;
    const int g0 = batched_gridder_shape(S), d0 = batched_degridder_shape(S);
    double best_g = 1e300, best_d = 1e300;
    *best_gridder = g0;
    *best_degridder = d0;
    for (int sh = 0; sh < gridder_fast_shapes(); ++sh) {
        set_batched_gridder_shape(S, sh);
        int rc = idg_gridder(params, IDG_VARIANT_BATCHED, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers,
                             visibilities, spheroidal, aterms, subgrids, stream); // warm-up
        if (rc) {
            set_batched_gridder_shape(S, g0);
            return rc;
        }
        IDG_CUDA(cudaEventRecord(ev.a, st));
        for (int r = 0; r < repeats; ++r)
            idg_gridder(params, IDG_VARIANT_BATCHED, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers,
                        visibilities, spheroidal, aterms, subgrids, stream);
        IDG_CUDA(cudaEventRecord(ev.b, st));
        float ms = 0;
        if (int rc2 = ev.elapsed_ms(&ms)) return rc2;
        gridder_ms[sh] = ms / repeats;
        if (gridder_ms[sh] < best_g) {
            best_g = gridder_ms[sh];
            *best_gridder = sh;
        }
    }
    // the shape in use before keeps its place unless another is more than 1 %
    // faster: sample timings of shapes that close flip from run to run
    if (g0 >= 0 && g0 < gridder_fast_shapes() && gridder_ms[g0] <= kKeepMargin * best_g) *best_gridder = g0;
    set_batched_gridder_shape(S, *best_gridder);
    for (int sh = 0; sh < degridder_fast_shapes(); ++sh) {
        set_batched_degridder_shape(S, sh);
        int rc = idg_degridder(params, IDG_VARIANT_BATCHED, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers,
                               visibilities_out, spheroidal, aterms, subgrids, stream);
        if (rc) {
            set_batched_degridder_shape(S, d0);
            return rc;
        }
        IDG_CUDA(cudaEventRecord(ev.a, st));
        for (int r = 0; r < repeats; ++r)
            idg_degridder(params, IDG_VARIANT_BATCHED, nr_subgrids, metadata, ext, nr_rows, uvw, wavenumbers,
                          visibilities_out, spheroidal, aterms, subgrids, stream);
        IDG_CUDA(cudaEventRecord(ev.b, st));
        float ms = 0;
        if (int rc2 = ev.elapsed_ms(&ms)) return rc2;
        degridder_ms[sh] = ms / repeats;
        if (degridder_ms[sh] < best_d) {
            best_d = degridder_ms[sh];
            *best_degridder = sh;
        }
    }
    if (d0 >= 0 && d0 < degridder_fast_shapes() && degridder_ms[d0] <= kKeepMargin * best_d) *best_degridder = d0;
    set_batched_degridder_shape(S, *best_degridder);
    return IDG_OK;
}

IDG_API int idg_measure_fp32_peak(double *flops_per_second) {
    if (!flops_per_second) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL output");
    cudaError_t e = measure_fp32_peak(flops_per_second);
    if (e != cudaSuccess) return cuda_fail(e, "fp32 peak microbenchmark");
    return IDG_OK;
}

} // extern "C"
