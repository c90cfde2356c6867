/*
 * idg_gb300.h -- C ABI of the GB300 Image-Domain Gridding (IDG) library.
 *
 * One process drives one GPU.  All entry points return an idg_status (0 = OK);
 * idg_last_error() returns the text of the calling thread's last failure.
 * Device pointers are plain CUDA device addresses; `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).  Nothing here takes or
 * returns a PyTorch type.
 *
 * Data layouts (row-major, last index fastest) are those of the reference's
 * gridding benchmark:
 *   uvw          [nr_rows][3]                  float (metres)           types.hpp:50-56
 *   wavenumbers  [nr_channels]                 float (rad / metre)
 *   visibilities [nr_rows][nr_channels][4]     complex64 (xx, xy, yx, yy) common_gridding.cuh:14-18
 *   spheroidal   [S][S]                        float (taper)
 *   aterms       [nr_aterms][nr_stations][S][S][4] complex64               common_gridding.cuh:20-26
 *   metadata     [nr_subgrids]                 idg_metadata (36 B)       types.hpp:17-25
 *   subgrids     [nr_subgrids][4][S][S]        complex64                 common_gridding.cuh:7-12
 *   grid         [nr_w_planes][4][G][G]        complex64                 types.hpp:526-543
 * A "row" is one (baseline, timestep); metadata.time_offset (minus the first
 * entry's baseline_offset, plus its own) selects a subgrid's first row
 * (gridding_benchmark.cpp:61).
 */
#ifndef IDG_GB300_H
#define IDG_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define IDG_API __declspec(dllexport)
#else
#define IDG_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define IDG_ABI_VERSION 4

typedef enum idg_status {
    IDG_OK = 0,
    IDG_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, layout or plan entry */
    IDG_ERR_CUDA = 2,             /* a CUDA runtime call failed (text in idg_last_error) */
    IDG_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed / over budget */
    IDG_ERR_UNSUPPORTED = 4,      /* shape outside what the kernels implement */
    IDG_ERR_TIMEOUT = 5,          /* a bounded wait expired */
    IDG_ERR_DEVICE_CHECK = 6,     /* a kernel's own bounds check rejected a plan entry */
    IDG_ERR_NOT_FOUND = 7,        /* unknown job id */
    IDG_ERR_REJECTED = 8          /* admission control refused a job */
} idg_status;

/* 36-byte subgrid plan entry: the reference's Metadata, field for field
 * (gridding/inc/types.hpp:7-25). */
typedef struct idg_metadata {
    int32_t baseline_offset;
    int32_t time_offset;
    int32_t nr_timesteps;
    int32_t aterm_index;
    uint32_t station1;
    uint32_t station2;
    int32_t x, y, z;
} idg_metadata;

/* Per-subgrid sidecar for uneven plans (no counterpart in the reference's
 * Metadata): the channel range [channel_begin, channel_end) the subgrid
 * covers.  NULL sidecar = all channels.  Subgrid size is uniform per call. */
typedef struct idg_subgrid_ext {
    int32_t channel_begin;
    int32_t channel_end;
} idg_subgrid_ext;

/* Flags for idg_params.flags */
#define IDG_FLAG_DEGRID_ATERM_REFCPU 0x1u /* degridder applies A1^H P A2 (degridding_benchmark.cpp:113)
                                             instead of the adjoint A1 P A2^H (degridding_benchmark.cu:56) */
#define IDG_FLAG_NO_TAPER 0x2u            /* gridder/degridder skip the spheroidal (the FFT applies it) */
#define IDG_FLAG_TEST_LOST_COPY 0x100u    /* tests only: the batched gridders and the grid FFT declare their
                                             first staged copy 16 bytes larger than what they copy, so its
                                             bounded wait (2 s) runs out: the kernel sets status bit 2 and
                                             stops, without faulting the GPU (see idg_device_status) */

/* Geometry and physics shared by all kernels of one call. */
typedef struct idg_params {
    int32_t grid_size;    /* G */
    int32_t subgrid_size; /* S (even, 8..64) */
    int32_t nr_channels;  /* C (1..1024): row length of `visibilities` */
    int32_t nr_stations;
    int32_t nr_aterms;    /* leading extent of `aterms` (the reference's ntimeslots) */
    int32_t nr_w_planes;  /* leading extent of `grid` (>= 1) */
    float image_size;     /* radians; the reference hard-codes 0.1F (gridding_benchmark.cpp:33) */
    float w_step;         /* wavelengths; the reference hard-codes 0 (gridding_benchmark.cpp:32) */
    uint32_t flags;       /* IDG_FLAG_* */
    int32_t reserved;
} idg_params;

/* The reference's benchmark_result (gridding/inc/common_gridding.h:5-12):
 * times in microseconds, bandwidths in bytes per microsecond, -1 = N/A. */
typedef struct idg_benchmark_result {
    double in_transfer_time;
    double out_transfer_time;
    double in_bandwidth;
    double out_bandwidth;
    double compute_time;
} idg_benchmark_result;

/* Kernel variants */
#define IDG_VARIANT_PLAIN 0   /* one CTA per subgrid, one sincos per pixel-visibility */
#define IDG_VARIANT_BATCHED 1 /* persistent CTAs over a cost-sorted work list, TMA-staged inputs */

/* ------------------------------------------------------------------ */
/* Library                                                            */
/* ------------------------------------------------------------------ */
IDG_API int idg_abi_version(void);
IDG_API const char *idg_last_error(void);
/* Reads and (if clear != 0) resets the device-side check word of the current
 * device: bit 0 = a plan entry named rows/stations/A-terms out of range,
 * bit 1 = a shape the kernel cannot handle, bit 2 = a staged copy did not
 * arrive within its time limit (the kernel stopped; its outputs are
 * incomplete).  Synchronises `stream`. */
IDG_API int idg_device_status(void *stream, uint32_t *status, int clear);

/* ------------------------------------------------------------------ */
/* Kernels on device-resident data (stream-ordered, asynchronous)      */
/* ------------------------------------------------------------------ */

/* Gridder: subgrids[s] = taper * (A1^H * sum_{t,c} V[t,c] e^{i phi} * A2).
 * Replaces kernel_gridder_v7 (gridding/src/gridding_benchmark.cu:231-246) and
 * the CPU loops of gridding_benchmark.cpp:56-166.  `ext` may be NULL. */
IDG_API int idg_gridder(const idg_params *params, int variant, int64_t nr_subgrids,
                        const idg_metadata *metadata, const idg_subgrid_ext *ext, int64_t nr_rows,
                        const float *uvw, const float *wavenumbers, const void *visibilities,
                        const float *spheroidal, const void *aterms, void *subgrids, void *stream);

/* The batched gridder (IDG_VARIANT_BATCHED of idg_gridder), for callers that
 * may not allocate device memory.  No counterpart in the reference.
 * idg_gridder() obtains its two scratch words (work counter, check word) with
 * cudaMalloc on first use; this entry point keeps them in a 256-byte static
 * device array of the library instead and calls no allocator.  Same arguments
 * and result as idg_gridder().  Limits: at most 2^30 subgrids; calls on one
 * device share the array, so calls whose kernels could overlap on the GPU
 * must be serialised by the caller; a rejected plan entry yields a zero
 * subgrid and sets a bit that idg_noalloc_status() reports.  The first call on
 * a device does a one-time set-up: it looks up the array's address and loads
 * the kernels (under CUDA's lazy loading a kernel is otherwise loaded at its
 * first launch, and loading takes device memory).  Make that first call --
 * with nr_subgrids = 0 it does the set-up alone -- before the caller's pool
 * takes the device memory and before any stream capture on that device. */
IDG_API int idg_gridder_noalloc(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                                const idg_subgrid_ext *ext, int64_t nr_rows, const float *uvw,
                                const float *wavenumbers, const void *visibilities, const float *spheroidal,
                                const void *aterms, void *subgrids, void *stream);
/* The check word of the last idg_gridder_noalloc() call on the current device
 * (bit 0: a plan entry named rows, stations, A-terms or channels out of range
 * and its subgrid was left zero), read after synchronising `stream`.  Each
 * call clears the word when it starts.  Allocates nothing.  No counterpart in
 * the reference. */
IDG_API int idg_noalloc_status(void *stream, uint32_t *status);

/* Degridder: V[t,c] = sum_pixels A(taper * subgrid) e^{-i phi}; writes only
 * the rows/channels the plan names.  Replaces kernel_degridder_v6
 * (gridding/src/degridding_benchmark.cu:106-203) and the CPU loops of
 * degridding_benchmark.cpp:58-181. */
IDG_API int idg_degridder(const idg_params *params, int variant, int64_t nr_subgrids,
                          const idg_metadata *metadata, const idg_subgrid_ext *ext, int64_t nr_rows,
                          const float *uvw, const float *wavenumbers, void *visibilities,
                          const float *spheroidal, const void *aterms, const void *subgrids, void *stream);

/* In-place batched subgrid FFT (S in {8,16,24,32,48,64}).
 * direction +1 (image -> uv, after gridding):
 *   F[j][i] = sum_{y,x} t P[y][x] exp(+2 pi i((j-S/2)(y-S/2+1/2) + (i-S/2)(x-S/2+1/2))/S)
 * direction -1 (uv -> image, before degridding): the adjoint, with the taper
 * applied after the transform.  `taper` may be NULL (t = 1).  No
 * normalisation: backward(forward(P)) = S^2 P.  No counterpart in the
 * reference (its upstream ska-sdp-idg-bench holds one; not vendored). */
IDG_API int idg_subgrid_fft(const idg_params *params, int64_t nr_subgrids, int direction,
                            const float *taper, void *subgrids, void *stream);

/* Adder: grid[z][pol][y+j][x+i] += F[s][pol][j][i] for cells inside the grid.
 * w-stacking: planes z = 0..W-1 hold w offsets (z + 1/2) w_step; an entry with
 * -W <= z < 0 (negative w) is added by Hermitian symmetry into plane -z-1 at
 * the mirrored cell (G - y - j, G - x - i), conjugated, with xy and yx
 * swapped.  Entries with z outside [-W, W) are skipped. */
IDG_API int idg_adder(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                      const void *subgrids, void *grid, void *stream);
/* The adder with a fixed summation order.  idg_adder() sums overlapping
 * footprints with floating-point atomics, so the last bits of the grid change
 * from run to run.  Bins made once from a plan's HOST metadata (the subgrids
 * of each 32 x 32-cell grid tile, in subgrid order, cut into chunks of 128)
 * let idg_adder_binned() add the same subgrids with plain loads and stores in
 * that order: the grid is the same, bit for bit, on every run.  Same
 * definition as idg_adder(), mirror rule included.  The bins keep a device
 * copy of the metadata and room for the partial tiles of tiles with more than
 * one chunk; idg_tile_bins_info() reports (work items, tiles with several
 * chunks, partial tiles, their bytes).  Calls with the same bins must not
 * overlap on the GPU (they share the partial tiles).  No counterpart in the
 * reference; its upstream adder is not vendored. */
typedef struct idg_tile_bins idg_tile_bins;
IDG_API int idg_tile_bins_create(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                                 idg_tile_bins **bins);
IDG_API int idg_tile_bins_destroy(idg_tile_bins *bins);
IDG_API int idg_tile_bins_info(const idg_tile_bins *bins, int64_t *sizes);
IDG_API int idg_adder_binned(const idg_tile_bins *bins, const void *subgrids, void *grid, void *stream);
/* Splitter: F[s][pol][j][i] = grid[z][pol][y+j][x+i] (0 outside); the
 * adder's mirror rule for -W <= z < 0. */
IDG_API int idg_splitter(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                         const void *grid, void *subgrids, void *stream);
/* The splitter and the backward subgrid FFT (direction -1, with `spheroidal`
 * or NULL) in one pass: the same subgrids, bit for bit, as idg_splitter
 * followed by idg_subgrid_fft, without writing and reading them in between.
 * subgrids must be 16-byte aligned.  idg_degrid_visibilities, plans and the
 * server's degridding jobs use it. */
IDG_API int idg_split_subgrid_fft(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                                  const void *grid, const float *spheroidal, void *subgrids, void *stream);

/* In-place 2-D FFT of every plane of grid[W][4][G][G] (G a power of two,
 * 64 <= G <= 8192), the imaging step around the path:
 *   direction -1 (uv -> image):
 *     out[y][x] = c[y] c[x] sum_{v,u} grid[v][u] exp(-2 pi i((u-G/2)(x-G/2) + (v-G/2)(y-G/2))/G)
 *   direction +1 (image -> uv): the adjoint (c applied before the transform).
 * `correction` is a DEVICE array of G floats (the separable grid correction,
 * e.g. the reciprocal of the taper's transform) or NULL (c = 1).  No
 * normalisation.  The first call for a (device, G) allocates and uploads a
 * twiddle table (so that call is not stream-capturable).  The reference
 * benchmarks this transform separately (fft/, heFFTe). */
IDG_API int idg_grid_fft(const idg_params *params, void *grid, int direction, const float *correction,
                         void *stream);

/* ------------------------------------------------------------------ */
/* The gridding / degridding steps on device-resident data             */
/* ------------------------------------------------------------------ */
/* Gridding step: gridder (no taper) -> subgrid FFT +1 with the taper ->
 * adder into `grid` (accumulates; zero it first for a fresh image).
 * `subgrids` is caller-provided work space [nr_subgrids][4][S][S] complex64.
 * The reference benchmark stops at the gridder; the FFT and adder complete
 * the step the way its upstream IDG pipeline does. */
IDG_API int idg_grid_visibilities(const idg_params *params, int variant, int64_t nr_subgrids,
                                  const idg_metadata *metadata, const idg_subgrid_ext *ext, int64_t nr_rows,
                                  const float *uvw, const float *wavenumbers, const void *visibilities,
                                  const float *spheroidal, const void *aterms, void *subgrids, void *grid,
                                  void *stream);
/* Degridding step: splitter from `grid` -> subgrid FFT -1 with the taper ->
 * degridder (no taper) into the rows/channels the plan names. */
IDG_API int idg_degrid_visibilities(const idg_params *params, int variant, int64_t nr_subgrids,
                                    const idg_metadata *metadata, const idg_subgrid_ext *ext, int64_t nr_rows,
                                    const float *uvw, const float *wavenumbers, void *visibilities,
                                    const float *spheroidal, const void *aterms, void *subgrids, const void *grid,
                                    void *stream);

/* ------------------------------------------------------------------ */
/* Planner: the subgrid plan from uvw, on the GPU                      */
/* ------------------------------------------------------------------ */
typedef struct idg_planner_params {
    int64_t nr_baselines;   /* rows of baseline b are b*nr_timesteps .. (b+1)*nr_timesteps-1 */
    int32_t nr_timesteps;   /* per baseline */
    int32_t nr_channels;
    int32_t subgrid_size;   /* S */
    int32_t grid_size;      /* G */
    int32_t max_timesteps;  /* per subgrid */
    int32_t aterm_interval; /* timesteps per A-term slot; 0 = one slot */
    int32_t margin;         /* cells of a subgrid kept free for the taper; usable width S - margin */
    int32_t nr_w_planes;    /* W (>= 1); used when w_step > 0 */
    double image_size;      /* radians */
    double w_step;          /* wavelengths; > 0: w-stacking, 0: every z = 0 */
} idg_planner_params;
/* uvw-driven plan with channel and time splitting: per baseline the channels
 * are cut into contiguous groups (a group closes before channel c when
 * reach * (f_c - f_first) > (S - margin) / 2, reach = the baseline's largest
 * |u| or |v| in cells per Hz); per group the time axis is walked and a
 * subgrid closed when the uv extent of its samples would exceed S - margin
 * cells, at max_timesteps, or at an A-term slot boundary; the subgrid's centre
 * cell sits on the centre of that extent; with w_step > 0 its w-plane is
 * z = floor(w_mid / w_step) (w_mid: centre of its w extent in wavelengths),
 * clipped to [-W, W-1], negative z being the adder's mirrored planes.  Inputs are DEVICE arrays: uvw
 * [nr_baselines * nr_timesteps][3] float (metres), frequencies [nr_channels]
 * double (Hz), baselines [nr_baselines][2] uint32 (stations).  Outputs:
 * `metadata` and `ext` (DEVICE, capacity max_subgrids) in (baseline, channel
 * group, time) order, and the count in *nr_subgrids (host); when the plan has
 * more than max_subgrids entries the call fails with the needed count in
 * *nr_subgrids.  Synchronises `stream`; allocates its work space with
 * cudaMallocAsync on `stream`.  The reference's plan is random
 * (gridding_initialization.cpp:158-182); this has no counterpart there. */
IDG_API int idg_plan_subgrids(const idg_planner_params *params, const float *uvw, const double *frequencies,
                              const uint32_t *baselines, int64_t max_subgrids, idg_metadata *metadata,
                              idg_subgrid_ext *ext, int64_t *nr_subgrids, void *stream);

/* ------------------------------------------------------------------ */
/* Execution plans (batching form): device-resident plan + CUDA graph  */
/* ------------------------------------------------------------------ */
/* A plan keeps a set of subgrids on the device: metadata, channel sidecar, a
 * work list ordering the subgrids longest first (uneven subgrids then finish
 * together in one persistent launch), the plan's own scheduler words, the
 * subgrid work space and the tile bins of its adder (idg_adder_binned: the
 * plan's grid is the same bit for bit on every run).  `metadata` and `ext` are HOST arrays, validated and
 * copied at creation.  The steps are those of idg_grid_visibilities /
 * idg_degrid_visibilities.  No counterpart in the reference. */
typedef struct idg_plan idg_plan;
IDG_API int idg_plan_create(const idg_params *params, int variant, int64_t nr_subgrids, const idg_metadata *metadata,
                            const idg_subgrid_ext *ext, int64_t nr_rows, idg_plan **plan);
IDG_API int idg_plan_destroy(idg_plan *plan);
/* Caps the persistent kernels of this plan at max_ctas CTAs (0 = fill the GPU),
 * so that several plans can share the GPU at the same time. */
IDG_API int idg_plan_set_cta_limit(idg_plan *plan, int max_ctas);
IDG_API int idg_plan_grid(idg_plan *plan, const float *uvw, const float *wavenumbers, const void *visibilities,
                          const float *spheroidal, const void *aterms, void *grid, void *stream);
IDG_API int idg_plan_degrid(idg_plan *plan, const float *uvw, const float *wavenumbers, void *visibilities,
                            const float *spheroidal, const void *aterms, const void *grid, void *stream);
/* Captures one imaging cycle on these device buffers -- zero `grid`, grid
 * `visibilities_in` into it, degrid it into `visibilities_out` -- as a CUDA
 * graph; idg_plan_launch_cycle() replays it with a single launch. */
IDG_API int idg_plan_capture_cycle(idg_plan *plan, const float *uvw, const float *wavenumbers,
                                   const void *visibilities_in, const float *spheroidal, const void *aterms, void *grid,
                                   void *visibilities_out);
IDG_API int idg_plan_launch_cycle(idg_plan *plan, void *stream);
/* Reads (and optionally clears) the plan's device check word; synchronises `stream`. */
IDG_API int idg_plan_status(idg_plan *plan, void *stream, uint32_t *status, int clear);

/* One imaging cycle over several plans that share one uv-grid -- typically one
 * plan per subgrid size of a job whose subgrids differ in size -- captured as a
 * single CUDA graph: zero `grid`, the gridding step of every plan in order,
 * then the degridding step of every plan.  Plans may differ in subgrid size and
 * channel count but must agree on grid_size and nr_w_planes.  Array arguments
 * hold one DEVICE pointer per plan (plan i reads uvw[i], wavenumbers[i],
 * visibilities_in[i], spheroidal[i], aterms[i] and writes visibilities_out[i]).
 * The buffers must stay allocated while the cycle is used.  No counterpart in
 * the reference. */
typedef struct idg_cycle idg_cycle;
IDG_API int idg_cycle_capture(int nr_plans, idg_plan *const *plans, const float *const *uvw,
                              const float *const *wavenumbers, const void *const *visibilities_in,
                              const float *const *spheroidal, const void *const *aterms, void *grid,
                              void *const *visibilities_out, idg_cycle **cycle);
IDG_API int idg_cycle_launch(idg_cycle *cycle, void *stream);
IDG_API int idg_cycle_destroy(idg_cycle *cycle);

/* ------------------------------------------------------------------ */
/* Serving: continuous batching of gridding / degridding jobs          */
/* ------------------------------------------------------------------ */
/* A server runs a scheduler thread that admits submitted jobs, in arrival
 * order, whenever one of `max_slots` slots (CUDA streams) is free and the
 * job's device footprint fits what `hbm_budget_bytes` leaves after the running
 * jobs (a job that cannot fit at all is rejected at submission; a job that
 * does not fit yet is overtaken by later jobs on other grids).  Admitted jobs
 * run concurrently: copies in, the batched kernels, copies out, each on its
 * slot's stream; with `cta_share` the persistent kernels of concurrently
 * running jobs split the SMs.  uv-grids are device-resident and owned by the
 * server; gridding jobs add into one, degridding jobs read one, and jobs of a
 * different kind on the same grid are ordered on the GPU.  Host buffers of a
 * job must stay valid until idg_server_wait() returns for it and should be
 * pinned (page-locked) for full copy bandwidth; every submitted job must be
 * waited on.  No counterpart in the reference. */
typedef struct idg_server idg_server;
typedef struct idg_server_config {
    int32_t max_slots;        /* jobs on the GPU at once (1..64) */
    int32_t cta_share;        /* nonzero: running jobs share the SMs between their persistent kernels */
    int64_t hbm_budget_bytes; /* device memory jobs may hold at once (resident grids not counted) */
} idg_server_config;

#define IDG_JOB_GRID 0
#define IDG_JOB_DEGRID 1
typedef struct idg_job {
    int32_t op;      /* IDG_JOB_GRID or IDG_JOB_DEGRID */
    int32_t variant; /* IDG_VARIANT_* */
    idg_params params;
    int64_t nr_subgrids;
    const idg_metadata *metadata; /* host */
    const idg_subgrid_ext *ext;   /* host, may be NULL */
    int64_t nr_rows;
    const float *uvw;         /* host [nr_rows][3] */
    const float *wavenumbers; /* host [C] */
    const void *vis_in;       /* host [nr_rows][C][4] complex64 (gridding jobs) */
    void *vis_out;            /* host [nr_rows][C][4] complex64 (degridding jobs) */
    const float *spheroidal;  /* host [S][S] */
    const void *aterms;       /* host [nr_aterms][stations][S][S][4] complex64 */
    int64_t grid_id;          /* a grid from idg_server_grid_create */
} idg_job;

typedef struct idg_job_stats {
    double queue_ms;   /* submission to admission */
    double run_ms;     /* admission to completion */
    double latency_ms; /* submission to completion */
    int64_t visibilities;
    int32_t status;
    int32_t reserved;
    /* Device interval of the job's kernels (first kernel queued .. last kernel
     * done), in ms since the server was created, from CUDA events on the job's
     * slot stream; -1 when not recorded.  Intervals of two jobs that intersect
     * show that their kernels ran on the GPU at the same time. */
    double device_start_ms;
    double device_end_ms;
    /* The job's whole stream work (its copies in, kernels and copy out), in
     * the same clock: stream_start_ms .. device_start_ms is the copy in plus
     * any wait for the grid's other jobs. */
    double stream_start_ms;
    double stream_end_ms;
} idg_job_stats;

typedef struct idg_server_stats {
    int64_t completed, rejected, failed, queued, running;
    int64_t hbm_in_use, hbm_peak;
    double p50_ms, p99_ms, mean_ms; /* job latency (submission to completion) over completed jobs */
    double mvis_per_s;              /* visibilities of completed jobs / (first submission .. last completion) */
} idg_server_summary;

IDG_API int idg_server_create(const idg_server_config *config, idg_server **server);
/* Finishes the queued and running jobs, then frees everything. */
IDG_API int idg_server_destroy(idg_server *server);
IDG_API int idg_server_grid_create(idg_server *server, int32_t grid_size, int32_t nr_w_planes, int64_t *grid_id);
/* Copies a grid to the host after every job on it that was submitted before
 * this call (it waits for them to be admitted, then for them to finish, on a
 * stream of its own; it returns when the copy is done).  Gridding jobs on that
 * grid are not admitted while the copy runs; degridding jobs may run beside
 * it. */
IDG_API int idg_server_grid_read(idg_server *server, int64_t grid_id, void *host_out);
/* Frees a grid; IDG_ERR_REJECTED while jobs are queued or running on it or a
 * read of it is in progress. */
IDG_API int idg_server_grid_release(idg_server *server, int64_t grid_id);
IDG_API int idg_server_submit(idg_server *server, const idg_job *job, int64_t *job_id);
/* Waits at most timeout_ms for a job (IDG_ERR_TIMEOUT otherwise); returns the job's status. */
IDG_API int idg_server_wait(idg_server *server, int64_t job_id, int64_t timeout_ms, idg_job_stats *stats);
IDG_API int idg_server_stats(idg_server *server, idg_server_summary *stats);

/* Timing of one host-buffer imaging cycle (milliseconds, bytes). */
typedef struct idg_cycle_timing {
    double total_ms;      /* first host-to-device copy issued .. last device-to-host copy done */
    double gridding_ms;   /* device time of the gridding phase (gridder + FFT + adder, all chunks) */
    double degridding_ms; /* device time of the degridding phase (splitter + FFT + degridder) */
    int64_t h2d_bytes;
    int64_t d2h_bytes;
    int64_t kernel_launches;
    /* The visibility copies alone: h2d_vis_ms and d2h_vis_ms are the sums of
     * the durations of the copies in and out (a copy in starts when the
     * stream reaches it, a copy out when its chunk is degridded).  bytes / ms
     * gives the host copy rate the cycle saw. */
    double h2d_vis_ms;
    double d2h_vis_ms;
    int64_t h2d_vis_bytes;
    int64_t d2h_vis_bytes;
    int64_t grid_chunks;   /* chunks of the gridding phase */
    int64_t degrid_chunks; /* chunks of the degridding phase */
    /* Time the gridding kernels spent waiting for their chunks' copies in
     * (within gridding_ms), and the growth ratio of the chunks. */
    double gridding_wait_ms;
    double chunk_ratio;
    /* From the call's first copy in to the end of this cycle's copies out
     * (idg_imaging_cycles; for idg_imaging_cycle it equals total_ms). */
    double end_ms;
    /* From this cycle's first copy in to the end of its last visibility copy
     * in: beside h2d_vis_ms, the time its copy stream spent on other copies
     * (plan, uvw, constants) or waiting. */
    double h2d_span_ms;
} idg_cycle_timing;

/* chunk_subgrids of idg_imaging_cycle: chunks sized for the copy pipeline */
#define IDG_CHUNKS_AUTO (-1)
/* ... with the growth ratio set from the previous cycle: at most 0.9 x
 * copy rate / kernel rate, stepped down by 15 % after a cycle whose gridding
 * kernels waited for copies more than 2 % of the phase and up by 5 % after
 * one that did not, kept within [1.1, 1.6].  Slower or unevenly arriving
 * copies get finer chunks.  The first cycle uses 1.6. */
#define IDG_CHUNKS_ADAPTIVE (-2)

/* One imaging cycle on HOST buffers: copies the plan, uvw, wavenumbers,
 * taper, A-terms and input visibilities in, grids them into a zeroed grid,
 * degrids the grid back into predicted visibilities and copies those out
 * (and the grid, if `grid_out` is not NULL).  Visibility copies are cut into
 * chunks on their own streams so that transfers overlap the kernels (the
 * plan's rows must then be in chunk order; otherwise the cycle runs as one
 * chunk).  chunk_subgrids > 0: chunks of that many subgrids; IDG_CHUNKS_AUTO:
 * ten chunks per phase whose sizes grow by 1.6x from chunk to chunk while
 * gridding (the first copy in is small, so the kernels start early, and each
 * later copy finishes while the previous chunk is gridded, for copy rates of
 * 1.6x the rate the kernels consume) and shrink by 1.6x while degridding (the
 * last copy out is small), at least 1024 subgrids each; IDG_CHUNKS_ADAPTIVE:
 * the same with the ratio learned from the previous cycle; 0: one chunk.  uvw
 * rows travel with their chunk.  Device buffers are kept between calls of
 * the same sizes and freed by idg_release_buffers().  Pinned host buffers
 * give full copy bandwidth.  The cycle clears the device check word (see
 * idg_device_status) before its first kernel and returns IDG_ERR_DEVICE_CHECK
 * when one of its own kernels set it.  Every return, an error included, comes
 * after all of the call's copies from and into the host buffers have ended. */
IDG_API int idg_imaging_cycle(const idg_params *params, int variant, int64_t nr_subgrids,
                              const idg_metadata *metadata, int64_t nr_rows, const float *uvw,
                              const float *wavenumbers, const void *visibilities_in, const float *spheroidal,
                              const void *aterms, void *visibilities_out, void *grid_out, int64_t chunk_subgrids,
                              idg_cycle_timing *timing);

/* One cycle of idg_imaging_cycles: its plan, uvw rows and visibilities on
 * host buffers, as idg_imaging_cycle takes them. */
typedef struct idg_cycle_io {
    int64_t nr_subgrids;
    const idg_metadata *metadata;
    int64_t nr_rows;
    const float *uvw;
    const void *visibilities_in;
    void *visibilities_out;
    void *grid_out;           /* may be NULL */
    idg_cycle_timing *timing; /* may be NULL */
} idg_cycle_io;

/* A run of imaging cycles on host buffers that share the wavenumbers, taper
 * and A-terms (copied in once), each cycle as idg_imaging_cycle runs it, with
 * the same outputs.  Cycle i+1's copies in (plan, uvw, visibilities) start as
 * soon as cycle i's gridding has started, each chunk of visibilities once
 * cycle i's gridding has read the rows it overwrites, and so run while cycle
 * i grids and degrids; cycle i's copies out run while it degrids and while
 * cycle i+1 grids.  With IDG_CHUNKS_AUTO / IDG_CHUNKS_ADAPTIVE the first
 * cycle's gridding and the last cycle's degridding have ten chunks, the other
 * phases four.  Because cycle i+1 reads its host inputs before cycle i has
 * written its outputs, no cycle may read host memory that an earlier cycle of
 * the call writes (IDG_ERR_INVALID_ARGUMENT; to feed one cycle's output to
 * the next, call idg_imaging_cycle per cycle).  Cycles may share their input
 * and output buffers.  Each cycle's timing reports its own copies and phases;
 * total_ms runs from its own first copy in, end_ms from the call's.  With
 * IDG_CHUNKS_ADAPTIVE the first cycle sets the ratio for the next call.  At
 * most 4096 cycles per call. */
IDG_API int idg_imaging_cycles(const idg_params *params, int variant, int64_t nr_cycles, const idg_cycle_io *cycles,
                               const float *wavenumbers, const float *spheroidal, const void *aterms,
                               int64_t chunk_subgrids);
IDG_API int idg_release_buffers(void);

/* ------------------------------------------------------------------ */
/* Drop-in launchers on host data                                      */
/* ------------------------------------------------------------------ */
/* The reference's per-call launcher configuration (the fields of
 * gridding/inc/gridding_configuration.h:54-65 that the launchers read). */
typedef struct idg_launch_config {
    int64_t niterations;
    int64_t grid_size;
    int64_t subgrid_size;
    int64_t nstations;
    int64_t nchannels;
    int64_t ntimeslots;
    int64_t ntimesteps_per_subgrid;
    float image_size; /* 0 = the reference's 0.1F */
    float w_step;     /* the reference's 0 */
    uint32_t flags;   /* IDG_FLAG_*; the launchers default to the reference CPU A-term convention
                         only when IDG_FLAG_DEGRID_ATERM_REFCPU is set */
    int32_t variant;  /* IDG_VARIANT_* */
} idg_launch_config;

/* Replaces gridding_benchmark_launcher<hardware_type::gpu>::launch
 * (gridding/inc/gridding_benchmark.h:10-21, gridding/src/gridding_benchmark.cu:248-361).
 * Host arrays in the reference's layouts (baselines [n_baselines][2] uint32,
 * frequencies [C] float, both unused by the kernels, may be NULL).  Copies the
 * inputs in, grids `niterations` times, copies the subgrids OUT into
 * `subgrids` (the reference copies them host-to-device at
 * gridding_benchmark.cu:345, which leaves the host array untouched), and
 * fills `result` with the reference's timing fields. */
IDG_API int idg_gridding_launch(const idg_launch_config *config, const float *uvw, const void *visibilities,
                                const uint32_t *baselines, const void *aterms, const float *frequencies,
                                const float *wavenumbers, const float *spheroidal, void *subgrids,
                                const idg_metadata *metadata, idg_benchmark_result *result);

/* Replaces degridding_benchmark_launcher<hardware_type::gpu>::launch
 * (gridding/inc/degridding_benchmark.h:18-28, gridding/src/degridding_benchmark.cu:205-318).
 * Copies the subgrids IN (the reference never does, degridding_benchmark.cu:255-264),
 * degrids, and copies the visibilities OUT into `visibilities`. */
IDG_API int idg_degridding_launch(const idg_launch_config *config, const float *uvw, void *visibilities,
                                  const uint32_t *baselines, const void *aterms, const float *frequencies,
                                  const float *wavenumbers, const float *spheroidal, const void *subgrids,
                                  const idg_metadata *metadata, idg_benchmark_result *result);

/* ------------------------------------------------------------------ */
/* Reference-compatible synthetic inputs and plan                     */
/* ------------------------------------------------------------------ */
/* Fills host buffers exactly as the reference's launch_gridding does before it
 * dispatches (srand(0); initialize_uvw, _frequencies, _wavenumbers,
 * _visibilities, _baselines, _spheroidal, _aterms, _metadata:
 * gridding/src/gridding_benchmark.cpp:203-213, gridding_initialization.cpp:7-182),
 * using the C library's rand().  image_size as passed (the reference: 0.1F). */
IDG_API int idg_reference_dataset(int64_t grid_size, int64_t subgrid_size, int64_t nstations, int64_t nchannels,
                                  int64_t ntimeslots, int64_t ntimesteps_per_subgrid, float image_size,
                                  float *uvw, float *frequencies, float *wavenumbers, void *visibilities,
                                  uint32_t *baselines, float *spheroidal, void *aterms, idg_metadata *metadata);

/* ------------------------------------------------------------------ */
/* Launch shapes of the batched kernels and their autotuner            */
/* ------------------------------------------------------------------ */
/* The batched gridder and degridder are compiled in several launch shapes
 * (threads per CTA, pixels, quads or octets per thread, staging tile, CTAs
 * per SM).  Until set here or by idg_autotune(), a subgrid size uses the
 * shapes measured fastest for it on GB300 (the mirror-quad kernels where
 * their layout fits the size).  No counterpart in the reference. */
IDG_API int idg_batched_shapes(int *gridder_shapes, int *degridder_shapes);
IDG_API int idg_set_batched_shapes(int subgrid_size, int gridder_shape, int degridder_shape);
IDG_API int idg_get_batched_shapes(int subgrid_size, int *gridder_shape, int *degridder_shape);
/* Times every shape of both batched kernels on the given (device) plan and
 * data -- writes `subgrids` and `visibilities_out` -- and selects the fastest
 * for params->subgrid_size on the current device; the shape in use before
 * keeps its place unless another is more than 1 % faster (sample timings of
 * shapes that close change from run to run).  gridder_ms / degridder_ms
 * receive the mean time of each shape (arrays of the sizes idg_batched_shapes
 * reports).  Synchronises `stream`. */
IDG_API int idg_autotune(const idg_params *params, int64_t nr_subgrids, const idg_metadata *metadata,
                         const idg_subgrid_ext *ext, int64_t nr_rows, const float *uvw, const float *wavenumbers,
                         const void *visibilities, const float *spheroidal, const void *aterms, void *subgrids,
                         void *visibilities_out, void *stream, int repeats, double *gridder_ms,
                         double *degridder_ms, int *best_gridder, int *best_degridder);

/* Reports the peak FP32 FMA rate of the current device measured by a short
 * dependent-chain microbenchmark (flop/s, 2 flop per FMA). */
IDG_API int idg_measure_fp32_peak(double *flops_per_second);

#ifdef __cplusplus
}
#endif
#endif /* IDG_GB300_H */
