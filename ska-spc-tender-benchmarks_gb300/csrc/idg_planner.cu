// idg_planner.cu -- the uvw-driven subgrid planner on the GPU.
//
// Same plan, bit for bit, as the host planner datasets.plan_subgrids_split:
//  1. per baseline (one warp): reach = max_t max(|u_t|, |v_t|) * scale, and the
//     channels cut into contiguous groups -- a group closes before channel c
//     when reach * (f_c - f_c0) > width / 2 (width = S - margin cells);
//  2. per (baseline, channel group) (one thread): the time axis is walked and
//     a subgrid closed when the uv extent of its samples (both edge channels,
//     all its timesteps) would exceed `width` cells, when it holds
//     max_timesteps steps, or at an A-term slot boundary; its corner puts the
//     centre cell on the centre of that extent;
//  3. the per-(baseline, group) counts are scanned on the host in (baseline,
//     group, time) order, and step 2 runs again writing the entries.
// All extents are FP64 with explicitly rounded operations (no contraction
// into FMA), in the host planner's order of evaluation, so that the integer
// corners come out identical.
#include <cmath>
#include <vector>

#include "idg_host.h"
#include "idg_internal.h"

namespace idg {

namespace {

struct PlanArgs {
    int64_t nb;
    int nt, C, S, G, tmax, ai, width, W;
    double scale, w_step;
    const float *uvw;        // [nb * nt][3]
    const double *f;         // [C] Hz
    const uint32_t *bl;      // [nb][2]
    int *groups_end;         // [nb][C]: end channel of each group
    int *ngroups;            // [nb]
    int *counts;             // [nb][C]: subgrids per (baseline, group)
    const int64_t *offsets;  // [nb][C]: first entry of each (baseline, group)
    idg_metadata *md;
    idg_subgrid_ext *ext;
};

constexpr double kSpeedOfLight = 299792458.0;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// Step 1: reach and channel groups, one warp per baseline.
__global__ void plan_groups_kernel(PlanArgs a) {
    const int64_t b = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (b >= a.nb) return;
    const float *p = a.uvw + 3 * (b * a.nt);
    double m = 0.0;
    for (int t = lane; t < a.nt; t += 32) m = fmax(m, fmax(fabs((double)p[3 * t]), fabs((double)p[3 * t + 1])));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane != 0) return;
    const double reach = mul(m, a.scale), half = 0.5 * (double)a.width;
    int c0 = 0, ng = 0;
    for (int c = 1; c <= a.C; ++c) {
        if (c == a.C || mul(reach, sub(a.f[c], a.f[c0])) > half) {
            a.groups_end[b * a.C + ng++] = c;
            c0 = c;
        }
    }
    a.ngroups[b] = ng;
}

// Per-timestep uv bounds of a group's two edge channels, in cells.
__device__ __forceinline__ void bounds(const float *row, double fa, double fb, double scale, double &lu, double &hu,
                                       double &lv, double &hv) {
    const double u = row[0], v = row[1];
    const double ua = mul(mul(u, fa), scale), ub = mul(mul(u, fb), scale);
    const double va = mul(mul(v, fa), scale), vb = mul(mul(v, fb), scale);
    lu = fmin(ua, ub);
    hu = fmax(ua, ub);
    lv = fmin(va, vb);
    hv = fmax(va, vb);
}

// Steps 2 and 3: walk one (baseline, group); WRITE = false counts, true emits.
template <bool WRITE>
__global__ void plan_walk_kernel(PlanArgs a) {
    const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= a.nb * a.C) return;
    const int64_t b = slot / a.C;
    const int g = (int)(slot - b * a.C);
    if (g >= a.ngroups[b]) {
        if (!WRITE) a.counts[slot] = 0;
        return;
    }
    const int c0 = g == 0 ? 0 : a.groups_end[b * a.C + g - 1], c1 = a.groups_end[b * a.C + g];
    const double fa = a.f[c0], fb = a.f[c1 - 1], width = (double)a.width;
    const float *rows = a.uvw + 3 * (b * a.nt);
    int64_t out = WRITE ? a.offsets[slot] : 0;
    int count = 0;
    int t0 = 0;
    while (t0 < a.nt) {
        int t1 = min(a.nt, t0 + a.tmax);
        if (a.ai > 0) t1 = min(t1, (t0 / a.ai + 1) * a.ai);
        double mnu = INFINITY, mxu = -INFINITY, mnv = INFINITY, mxv = -INFINITY;
        int n = t1 - t0;
        for (int t = t0; t < t1; ++t) {
            double lu, hu, lv, hv;
            bounds(rows + 3 * t, fa, fb, a.scale, lu, hu, lv, hv);
            mnu = fmin(mnu, lu);
            mxu = fmax(mxu, hu);
            mnv = fmin(mnv, lv);
            mxv = fmax(mxv, hv);
            if (fmax(sub(mxu, mnu), sub(mxv, mnv)) > width) {
                n = t - t0;
                break;
            }
        }
        n = max(n, 1);
        if (WRITE) {
            double lu_min = INFINITY, hu_max = -INFINITY, lv_min = INFINITY, hv_max = -INFINITY;
            double lw_min = INFINITY, hw_max = -INFINITY;
            for (int t = t0; t < t0 + n; ++t) {
                double lu, hu, lv, hv;
                bounds(rows + 3 * t, fa, fb, a.scale, lu, hu, lv, hv);
                lu_min = fmin(lu_min, lu);
                hu_max = fmax(hu_max, hu);
                lv_min = fmin(lv_min, lv);
                hv_max = fmax(hv_max, hv);
                const double w = rows[3 * t + 2];
                const double wa = __ddiv_rn(mul(w, fa), kSpeedOfLight), wb = __ddiv_rn(mul(w, fb), kSpeedOfLight);
                lw_min = fmin(lw_min, fmin(wa, wb));
                hw_max = fmax(hw_max, fmax(wa, wb));
            }
            int z = 0;
            if (a.w_step > 0.0) {
                const double zf = floor(__ddiv_rn(mul(0.5, add(lw_min, hw_max)), a.w_step));
                z = (int)fmin(fmax(zf, (double)-a.W), (double)(a.W - 1));
            }
            const double mid_u = mul(0.5, add(lu_min, hu_max)), mid_v = mul(0.5, add(lv_min, hv_max));
            const double hg = 0.5 * (double)a.G, hs = 0.5 * (double)a.S;
            idg_metadata m;
            m.baseline_offset = 0;
            m.time_offset = (int32_t)(b * a.nt + t0);
            m.nr_timesteps = n;
            m.aterm_index = a.ai > 0 ? t0 / a.ai : 0;
            m.station1 = a.bl[2 * b];
            m.station2 = a.bl[2 * b + 1];
            m.x = (int32_t)floor(add(sub(add(mid_u, hg), hs), 0.5));
            m.y = (int32_t)floor(add(sub(add(mid_v, hg), hs), 0.5));
            m.z = z;
            a.md[out] = m;
            a.ext[out] = idg_subgrid_ext{c0, c1};
            ++out;
        }
        ++count;
        t0 += n;
    }
    if (!WRITE) a.counts[slot] = count;
}

} // namespace

extern "C" {

IDG_API int idg_plan_subgrids(const idg_planner_params *p, const float *uvw, const double *frequencies,
                              const uint32_t *baselines, int64_t max_subgrids, idg_metadata *metadata,
                              idg_subgrid_ext *ext, int64_t *nr_subgrids, void *stream) {
    if (!p || !nr_subgrids) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL argument");
    *nr_subgrids = 0;
    if (p->nr_baselines < 1 || p->nr_timesteps < 1 || p->nr_channels < 1 || p->subgrid_size < 2 ||
        p->grid_size < p->subgrid_size || p->max_timesteps < 1 || p->aterm_interval < 0 || p->margin < 0 ||
        p->margin >= p->subgrid_size || !(p->image_size > 0.0) || !(p->w_step >= 0.0) || p->nr_w_planes < 1)
        return fail(IDG_ERR_INVALID_ARGUMENT, "planner parameters out of range");
    if ((int64_t)p->nr_baselines * p->nr_timesteps > INT32_MAX)
        return fail(IDG_ERR_INVALID_ARGUMENT, "more than 2^31 rows");
    if (!uvw || !frequencies || !baselines) return fail(IDG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t nb = p->nr_baselines, slots = nb * p->nr_channels;
    PlanArgs a{};
    a.nb = nb;
    a.nt = p->nr_timesteps;
    a.C = p->nr_channels;
    a.S = p->subgrid_size;
    a.G = p->grid_size;
    a.tmax = p->max_timesteps;
    a.ai = p->aterm_interval;
    a.width = p->subgrid_size - p->margin;
    a.scale = p->image_size / kSpeedOfLight;
    a.w_step = p->w_step;
    a.W = p->nr_w_planes;
    a.uvw = uvw;
    a.f = frequencies;
    a.bl = baselines;
    // work space: offsets (int64) first, then group ends, counts and group counts
    void *work = nullptr;
    const size_t bytes = sizeof(int64_t) * (size_t)slots + sizeof(int) * (size_t)(2 * slots + nb);
    IDG_CUDA(cudaMallocAsync(&work, bytes, st));
    int64_t *d_off = static_cast<int64_t *>(work);
    a.offsets = d_off;
    a.groups_end = reinterpret_cast<int *>(d_off + slots);
    a.counts = a.groups_end + slots;
    a.ngroups = a.counts + slots;
    a.md = metadata;
    a.ext = ext;
    int rc = IDG_OK;
    cudaError_t e = cudaSuccess;
    std::vector<int> counts(slots);
    std::vector<int64_t> offs(slots);
    int64_t total = 0;
    do {
        plan_groups_kernel<<<(unsigned)((nb + 7) / 8), 256, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        plan_walk_kernel<false><<<(unsigned)((slots + 127) / 128), 128, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(counts.data(), a.counts, sizeof(int) * slots, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
        for (int64_t i = 0; i < slots; ++i) {
            offs[i] = total;
            total += counts[i];
        }
        *nr_subgrids = total;
        if (total > max_subgrids || total > INT32_MAX) {
            rc = fail(IDG_ERR_INVALID_ARGUMENT, "the plan has %lld subgrids, more than max_subgrids = %lld",
                      (long long)total, (long long)max_subgrids);
            break;
        }
        if (!metadata || !ext) {
            rc = fail(IDG_ERR_INVALID_ARGUMENT, "metadata / ext output is NULL");
            break;
        }
        if ((e = cudaMemcpyAsync(d_off, offs.data(), sizeof(int64_t) * slots, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        plan_walk_kernel<true><<<(unsigned)((slots + 127) / 128), 128, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        e = cudaStreamSynchronize(st);
    } while (false);
    cudaFreeAsync(work, st);
    cudaStreamSynchronize(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "GPU planner");
    return IDG_OK;
}

} // extern "C"

} // namespace idg
