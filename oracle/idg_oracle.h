/*
 * idg_oracle.h -- CPU oracle for the Image-Domain Gridding (IDG) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This restatement is the checker used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline / reference arm of bench.py.
 * Nothing in the shipped library links, loads or calls it.
 *
 * Pinning: the float variants follow the reference's CPU launchers operation
 * by operation (gridding/src/gridding_benchmark.cpp:56-166,
 * gridding/src/degridding_benchmark.cpp:58-181) and are compared bit for bit
 * against the reference compiled from its own sources (oracle/Makefile,
 * target `ref`) through the golden fixtures in tests/golden/.  The double
 * variants are the same loops in FP64 and serve as the precision oracle.
 * The subgrid FFT, adder and splitter have no counterpart in the reference
 * ("parity unpinned" at reference level): they are pinned against the
 * defining DFT sums evaluated directly in FP64.
 */
#ifndef IDG_ORACLE_H
#define IDG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 36-byte subgrid plan entry; field order and sizes follow
 * gridding/inc/types.hpp:7-25 (Coordinate, Baseline, Metadata). */
typedef struct {
    int32_t baseline_offset;
    int32_t time_offset;
    int32_t nr_timesteps;
    int32_t aterm_index;
    uint32_t station1;
    uint32_t station2;
    int32_t x, y, z;
} oracle_metadata;

/* Degridder A-term conventions.
 * ORACLE_ATERM_REFCPU : P' = A1^H * P * A2  (degridding_benchmark.cpp:113)
 * ORACLE_ATERM_ADJOINT: P' = A1 * P * A2^H  (degridding_benchmark.cu:56,
 *                       common_gridding.cuh:82-94; the adjoint of the gridder) */
enum { ORACLE_ATERM_REFCPU = 0, ORACLE_ATERM_ADJOINT = 1 };

typedef struct {
    int grid_size;
    int subgrid_size;
    int nr_channels;
    int nr_stations;
    int nr_subgrids;
    float image_size;   /* radians; the reference hard-codes 0.1F */
    float w_step;       /* wavelengths; the reference hard-codes 0 */
} oracle_params;

/* Gridder.  Inputs:
 *   uvw        [*][3] float (u, v, w in metres), row = time index
 *   wavenumbers[C] float (rad / metre)
 *   vis        [*][C][4] complex float, interleaved (re, im)
 *   spheroidal [S][S] float
 *   aterms     [nr_aterms][nr_stations][S][S][4] complex float
 *   metadata   [N]
 * Output subgrids [N][4][S][S] complex (float or double). */
void oracle_gridder_f32(const oracle_params *p, const float *uvw, const float *wavenumbers,
                        const float *vis, const float *spheroidal, const float *aterms,
                        const oracle_metadata *metadata, float *subgrids);
void oracle_gridder_f64(const oracle_params *p, const float *uvw, const float *wavenumbers,
                        const float *vis, const float *spheroidal, const float *aterms,
                        const oracle_metadata *metadata, double *subgrids);

/* Degridder: subgrids [N][4][S][S] complex float in, vis [*][C][4] out.
 * Only the rows named by the metadata are written. */
void oracle_degridder_f32(const oracle_params *p, int aterm_mode, const float *uvw,
                          const float *wavenumbers, const float *subgrids, const float *spheroidal,
                          const float *aterms, const oracle_metadata *metadata, float *vis);
void oracle_degridder_f64(const oracle_params *p, int aterm_mode, const float *uvw,
                          const float *wavenumbers, const float *subgrids, const float *spheroidal,
                          const float *aterms, const oracle_metadata *metadata, double *vis);

/* Subgrid DFT, evaluated directly (O(S^4) per subgrid) in FP64.
 * direction +1 (image -> uv, gridding side):
 *   F[j][i] = sum_{y,x} t(y,x) P[y][x] exp(+2 pi i ((j-S/2)(y-S/2+1/2) + (i-S/2)(x-S/2+1/2)) / S)
 * direction -1 (uv -> image, degridding side):
 *   P[y][x] = t(y,x) sum_{j,i} F[j][i] exp(-2 pi i (...) / S)
 * t is the taper when `taper` is non-NULL, else 1.  No normalisation: the
 * two directions are adjoint and backward(forward(P)) = S^2 P for t = 1.
 * Data are complex double [N][4][S][S]; in and out may not alias. */
void oracle_subgrid_dft_f64(int nr_subgrids, int subgrid_size, int direction, const float *taper,
                            const double *in, double *out);

/* Adder: grid[z][pol][y0+j][x0+i] += F[s][pol][j][i] for every cell inside
 * the G x G grid (cells outside are dropped), in subgrid order; z is the
 * metadata w-plane index.  An entry with -W <= z < 0 (negative w) adds
 * conj(F) to plane -z-1 at the mirrored cell (G - y0 - j, G - x0 - i) with
 * xy and yx swapped (Hermitian symmetry); entries with z outside [-W, W) are
 * skipped.  grid is complex double [W][4][G][G]. */
void oracle_adder_f64(int nr_subgrids, int subgrid_size, int grid_size, int nr_w_planes,
                      const oracle_metadata *metadata, const double *subgrids, double *grid);
/* Splitter: F[s][pol][j][i] = grid[z][pol][y0+j][x0+i], 0 outside; the
 * adder's mirror rule for -W <= z < 0 (conjugated read of the mirrored cell). */
void oracle_splitter_f64(int nr_subgrids, int subgrid_size, int grid_size, int nr_w_planes,
                         const oracle_metadata *metadata, const double *grid, double *subgrids);

/* The reference's CPU launchers in one call each (float, same loops), with
 * OpenMP over the pixels of each subgrid and over (time, channel) in the
 * degridder, as at gridding_benchmark.cpp:88 and degridding_benchmark.cpp:79,137.
 * Used as the timed CPU baseline ("port") where the reference itself cannot
 * be built.  Returns the number of OpenMP threads used. */
int oracle_cpu_gridding_omp(const oracle_params *p, const float *uvw, const float *wavenumbers,
                            const float *vis, const float *spheroidal, const float *aterms,
                            const oracle_metadata *metadata, float *subgrids);
int oracle_cpu_degridding_omp(const oracle_params *p, const float *uvw, const float *wavenumbers,
                              const float *subgrids, const float *spheroidal, const float *aterms,
                              const oracle_metadata *metadata, float *vis);
int oracle_omp_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
