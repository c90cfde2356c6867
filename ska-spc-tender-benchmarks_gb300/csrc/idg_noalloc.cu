// idg_noalloc.cu -- the batched gridder for callers that may not allocate
// device memory.
//
// The batched gridder needs two words of device scratch: the work counter its
// persistent CTAs pull subgrids from, and the check word it flags bad plan
// entries in.  idg_gridder() keeps those words in memory the library obtains
// with cudaMalloc on first use.  Some callers cannot allow that: a host
// application that has reserved all device memory through its own pool, a
// framework that forbids allocations outside its allocator, or a real-time
// loop that must not allocate once it is running.  idg_gridder_noalloc() runs
// the same kernel with its scratch in the file-scope array below instead, so
// the call itself allocates nothing; the caller passes every input and output.
//
// The array is g_noalloc_scratch: 256 bytes, loaded with the library on every
// device that uses it and kept until the process exits.  Word 0 is the work
// counter, word 1 the check word.  Each call clears both on the caller's
// stream before the launch.  All calls on a device share the array, so calls
// whose kernels overlap on the GPU (other streams, no ordering between them)
// race on the work counter and must be serialised by the caller.  A plan
// entry the kernel rejects yields an all-zero subgrid and sets bit 0 of the
// check word, which idg_noalloc_status() reads (idg_device_status() reports
// the other entry points' word only).
// The first call on a device does a one-time set-up there: it looks up the
// array's device address and loads the batched gridder's kernels into the
// context.  Under CUDA's lazy module loading both would otherwise happen at
// first use, and loading a module takes device memory -- which fails in the
// very case this entry point is for, a pool that already owns all of it.
// So make the first call on a device before the caller's pool takes the
// device memory, and before any stream capture on that device; a call with
// nr_subgrids = 0 does the set-up alone.
#include <mutex>
#include <vector>

#include "idg_device.cuh"
#include "idg_host.h"
#include "idg_internal.h"

namespace {

constexpr int kScratchWords = 64; // 256 bytes
// The work counter is a 32-bit integer that every CTA advances once past the
// last subgrid; plans are limited so that it cannot overflow.
constexpr int64_t kMaxSubgrids = int64_t(1) << 30;

static __device__ __align__(256) unsigned int g_noalloc_scratch[kScratchWords];

std::mutex g_addr_mutex;
std::vector<void *> g_addr; // per device: address of g_noalloc_scratch

// Set-up, once per device, with that device current: fetch the array's device
// address (host code cannot use the symbol itself as a pointer) and load the
// kernels this entry point launches.
int scratch_address(void **out) {
    int dev = 0;
    IDG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if ((int)g_addr.size() <= dev) g_addr.resize(dev + 1, nullptr);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return idg::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        e = idg::load_gridder_fast();
        if (e != cudaSuccess) return idg::cuda_fail(e, "loading the batched gridder's kernels");
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return IDG_OK;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

} // namespace

extern "C" IDG_API int idg_gridder_noalloc(const idg_params *params, int64_t nr_subgrids,
                                           const idg_metadata *metadata, const idg_subgrid_ext *ext,
                                           int64_t nr_rows, const float *uvw, const float *wavenumbers,
                                           const void *visibilities, const float *spheroidal, const void *aterms,
                                           void *subgrids, void *stream) {
    using namespace idg;
    if (int rc = check_params(params)) return rc;
    if (nr_subgrids < 0) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_subgrids %lld < 0", (long long)nr_subgrids);
    if (nr_subgrids > kMaxSubgrids)
        return fail(IDG_ERR_UNSUPPORTED,
                    "nr_subgrids %lld exceeds %lld, the most the allocation-free gridder's 32-bit work counter "
                    "can schedule",
                    (long long)nr_subgrids, (long long)kMaxSubgrids);
    void *scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    if (nr_subgrids == 0) return IDG_OK;
    if (nr_rows < 0) return fail(IDG_ERR_INVALID_ARGUMENT, "nr_rows %lld < 0", (long long)nr_rows);
    if (!metadata || !uvw || !wavenumbers || !visibilities || !aterms || !subgrids)
        return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (!spheroidal && !(params->flags & IDG_FLAG_NO_TAPER))
        return fail(IDG_ERR_INVALID_ARGUMENT, "spheroidal is NULL and IDG_FLAG_NO_TAPER is not set");
    if (!aligned16(visibilities) || !aligned16(aterms) || !aligned16(subgrids))
        return fail(IDG_ERR_INVALID_ARGUMENT, "visibilities, aterms and subgrids must be 16-byte aligned");

    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    IDG_CUDA(cudaMemsetAsync(scratch, 0, 2 * sizeof(unsigned int), st));

    KernelArgs a{};
    a.G = params->grid_size;
    a.S = params->subgrid_size;
    a.C = params->nr_channels;
    a.nr_stations = params->nr_stations;
    a.nr_aterms = params->nr_aterms;
    a.nr_w_planes = params->nr_w_planes > 0 ? params->nr_w_planes : 1;
    a.image_size = params->image_size;
    a.w_step = params->w_step;
    a.flags = params->flags;
    a.nr_subgrids = nr_subgrids;
    a.nr_rows = nr_rows;
    a.md = metadata;
    a.ext = ext;
    a.uvw = uvw;
    a.wavenumbers = wavenumbers;
    a.taper = spheroidal;
    a.aterms = reinterpret_cast<const float4 *>(aterms);
    a.vis = reinterpret_cast<float4 *>(const_cast<void *>(visibilities));
    a.subgrids = reinterpret_cast<float2 *>(subgrids);
    a.work_counter = reinterpret_cast<int *>(scratch);
    a.status = reinterpret_cast<unsigned *>(scratch) + 1;
    cudaError_t e = launch_gridder_fast(a, st, batched_gridder_shape(a.S));
    if (e != cudaSuccess) return cuda_fail(e, "allocation-free gridder launch");
    return IDG_OK;
}

extern "C" IDG_API int idg_noalloc_status(void *stream, uint32_t *status) {
    using namespace idg;
    if (!status) return fail(IDG_ERR_INVALID_ARGUMENT, "status is NULL");
    void *scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    IDG_CUDA(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
    unsigned word = 0;
    IDG_CUDA(cudaMemcpy(&word, reinterpret_cast<unsigned *>(scratch) + 1, sizeof word, cudaMemcpyDeviceToHost));
    *status = word;
    return IDG_OK;
}
