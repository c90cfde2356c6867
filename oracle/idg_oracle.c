/*
 * idg_oracle.c -- CPU oracle for the IDG hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm may load this code, and only as the checker or as the timed
 * CPU baseline.  The shipped library never calls it.
 *
 * The float functions restate the reference's CPU launchers operation for
 * operation so that, built with -ffp-contract=off against the same libm,
 * they reproduce the reference's bits:
 *   gridder   : gridding/src/gridding_benchmark.cpp:56-166
 *   degridder : gridding/src/degridding_benchmark.cpp:58-181
 *   l, m, n   : gridding/inc/math.hpp:20-37
 *   A-terms   : gridding/inc/math.hpp:39-100 (A1^H P A2), and the GPU
 *               degridder's A1 P A2^H (gridding/inc/common_gridding.cuh:82-94)
 * The double functions evaluate the same sums in FP64 from the same float
 * inputs; they are the precision oracle for the GPU kernels.
 */
#include "idg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* float complex helpers with the operation order GCC uses for        */
/* std::complex<float> (ac - bd, ad + bc), no FMA contraction.        */
/* ------------------------------------------------------------------ */
typedef struct { float re, im; } cf32;
typedef struct { double re, im; } cf64;

static inline cf32 cmul32(cf32 a, cf32 b) {
    cf32 r;
    float ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
    r.re = ac - bd;
    r.im = ad + bc;
    return r;
}
static inline cf32 cadd32(cf32 a, cf32 b) { cf32 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf32 conj32(cf32 a) { cf32 r = {a.re, -a.im}; return r; }

static inline cf64 cmul64(cf64 a, cf64 b) {
    cf64 r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cf64 cadd64(cf64 a, cf64 b) { cf64 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf64 conj64(cf64 a) { cf64 r = {a.re, -a.im}; return r; }

/* 2x2 complex matrix product c = a * b, row-major {xx, xy, yx, yy}, with the
 * accumulation order of math.hpp:44-54 (products of column 0, then += column 1). */
static void matmul32(const cf32 *a, const cf32 *b, cf32 *c) {
    c[0] = cmul32(a[0], b[0]);
    c[1] = cmul32(a[0], b[1]);
    c[2] = cmul32(a[2], b[0]);
    c[3] = cmul32(a[2], b[1]);
    c[0] = cadd32(c[0], cmul32(a[1], b[2]));
    c[1] = cadd32(c[1], cmul32(a[1], b[3]));
    c[2] = cadd32(c[2], cmul32(a[3], b[2]));
    c[3] = cadd32(c[3], cmul32(a[3], b[3]));
}
static void hermitian32(const cf32 *a, cf32 *b) {
    b[0] = conj32(a[0]);
    b[1] = conj32(a[2]);
    b[2] = conj32(a[1]);
    b[3] = conj32(a[3]);
}
static void matmul64(const cf64 *a, const cf64 *b, cf64 *c) {
    c[0] = cadd64(cmul64(a[0], b[0]), cmul64(a[1], b[2]));
    c[1] = cadd64(cmul64(a[0], b[1]), cmul64(a[1], b[3]));
    c[2] = cadd64(cmul64(a[2], b[0]), cmul64(a[3], b[2]));
    c[3] = cadd64(cmul64(a[2], b[1]), cmul64(a[3], b[3]));
}
static void hermitian64(const cf64 *a, cf64 *b) {
    b[0] = conj64(a[0]);
    b[1] = conj64(a[2]);
    b[2] = conj64(a[1]);
    b[3] = conj64(a[3]);
}

/* P <- A1^H P A2 (math.hpp:90-100) */
static void aterm_gridder32(cf32 *pix, const cf32 *a1, const cf32 *a2) {
    cf32 a1h[4], tmp[4];
    hermitian32(a1, a1h);
    matmul32(a1h, pix, tmp);
    matmul32(tmp, a2, pix);
}
/* P <- A1 P A2^H (common_gridding.cuh:82-94) */
static void aterm_degridder32(cf32 *pix, const cf32 *a1, const cf32 *a2) {
    cf32 a2h[4], tmp[4];
    matmul32(a1, pix, tmp);
    hermitian32(a2, a2h);
    matmul32(tmp, a2h, pix);
}
static void aterm_gridder64(cf64 *pix, const cf64 *a1, const cf64 *a2) {
    cf64 a1h[4], tmp[4];
    hermitian64(a1, a1h);
    matmul64(a1h, pix, tmp);
    matmul64(tmp, a2, pix);
}
static void aterm_degridder64(cf64 *pix, const cf64 *a1, const cf64 *a2) {
    cf64 a2h[4], tmp[4];
    matmul64(a1, pix, tmp);
    hermitian64(a2, a2h);
    matmul64(tmp, a2h, pix);
}

/* math.hpp:20-37, float */
static inline float compute_l32(int x, int S, float image_size) {
    return ((float)x + 0.5F - ((float)S / 2.F)) * image_size / (float)S;
}
static inline float compute_n32(float l, float m) {
    const float tmp = (l * l) + (m * m);
    return tmp > 1.F ? 1.F : tmp / (1.f + sqrtf(1.F - tmp));
}
static inline double compute_l64(int x, int S, double image_size) {
    return ((double)x + 0.5 - (double)S / 2.0) * image_size / (double)S;
}
static inline double compute_n64(double l, double m) {
    const double tmp = l * l + m * m;
    return tmp > 1.0 ? 1.0 : tmp / (1.0 + sqrt(1.0 - tmp));
}

static const float PI_F32 = (float)3.141592653589793; /* math.hpp:15-18 */

static inline size_t aterm_offset(const oracle_params *p, int aterm_index, unsigned station) {
    const size_t S = (size_t)p->subgrid_size;
    return ((size_t)aterm_index * (size_t)p->nr_stations + station) * S * S * 4;
}

/* ------------------------------------------------------------------ */
/* Gridder                                                            */
/* ------------------------------------------------------------------ */
void oracle_gridder_f32(const oracle_params *p, const float *uvw, const float *wavenumbers,
                        const float *vis, const float *spheroidal, const float *aterms,
                        const oracle_metadata *metadata, float *subgrids) {
    const int S = p->subgrid_size, C = p->nr_channels;
    const float image_size = p->image_size;
    const int baseline_offset_1 = metadata[0].baseline_offset;
    const cf32 *vis_c = (const cf32 *)vis;
    const cf32 *aterms_c = (const cf32 *)aterms;
    cf32 *sub_c = (cf32 *)subgrids;

    for (int s = 0; s < p->nr_subgrids; ++s) {
        const oracle_metadata md = metadata[s];
        const int time_offset = (md.baseline_offset - baseline_offset_1) + md.time_offset;
        const float w_offset_in_lambda = (float)((double)p->w_step * (md.z + 0.5));
        const float half_subgrid_size = (float)S * 0.5F;
        const float half_grid_size = (float)p->grid_size * 0.5F;
        const float u_offset = ((float)md.x + half_subgrid_size - half_grid_size) * (2.F * PI_F32 / image_size);
        const float v_offset = ((float)md.y + half_subgrid_size - half_grid_size) * (2.F * PI_F32 / image_size);
        const float w_offset = 2.F * PI_F32 * w_offset_in_lambda;
        const cf32 *a1 = aterms_c + aterm_offset(p, md.aterm_index, md.station1);
        const cf32 *a2 = aterms_c + aterm_offset(p, md.aterm_index, md.station2);

#ifdef _OPENMP
#pragma omp parallel for collapse(2)
#endif
        for (int y = 0; y < S; ++y) {
            for (int x = 0; x < S; ++x) {
                cf32 pix[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                const float l = compute_l32(x, S, image_size);
                const float m = compute_l32(y, S, image_size);
                const float n = compute_n32(l, m);
                for (int t = 0; t < md.nr_timesteps; ++t) {
                    const float *uvw_t = uvw + 3 * (size_t)(time_offset + t);
                    const float phase_index = uvw_t[0] * l + uvw_t[1] * m + uvw_t[2] * n;
                    const float phase_offset = u_offset * l + v_offset * m + w_offset * n;
                    for (int c = 0; c < C; ++c) {
                        const float phase = phase_offset - (phase_index * wavenumbers[c]);
                        const cf32 phasor = {cosf(phase), sinf(phase)};
                        const cf32 *v = vis_c + ((size_t)(time_offset + t) * C + c) * 4;
                        for (int pol = 0; pol < 4; ++pol) pix[pol] = cadd32(pix[pol], cmul32(v[pol], phasor));
                    }
                }
                const size_t px = ((size_t)y * S + x) * 4;
                aterm_gridder32(pix, a1 + px, a2 + px);
                const float sph = spheroidal[y * S + x];
                for (int pol = 0; pol < 4; ++pol) {
                    cf32 *dst = sub_c + (((size_t)s * 4 + pol) * S + y) * S + x;
                    dst->re = pix[pol].re * sph;
                    dst->im = pix[pol].im * sph;
                }
            }
        }
    }
}

void oracle_gridder_f64(const oracle_params *p, const float *uvw, const float *wavenumbers,
                        const float *vis, const float *spheroidal, const float *aterms,
                        const oracle_metadata *metadata, double *subgrids) {
    const int S = p->subgrid_size, C = p->nr_channels;
    const double image_size = p->image_size;
    const int baseline_offset_1 = metadata[0].baseline_offset;
    const cf32 *vis_c = (const cf32 *)vis;
    const cf32 *aterms_c = (const cf32 *)aterms;
    cf64 *sub_c = (cf64 *)subgrids;

    for (int s = 0; s < p->nr_subgrids; ++s) {
        const oracle_metadata md = metadata[s];
        const int time_offset = (md.baseline_offset - baseline_offset_1) + md.time_offset;
        const double u_offset = ((double)md.x + S / 2.0 - p->grid_size / 2.0) * (2.0 * M_PI / image_size);
        const double v_offset = ((double)md.y + S / 2.0 - p->grid_size / 2.0) * (2.0 * M_PI / image_size);
        const double w_offset = 2.0 * M_PI * (double)p->w_step * (md.z + 0.5);
        const cf32 *a1 = aterms_c + aterm_offset(p, md.aterm_index, md.station1);
        const cf32 *a2 = aterms_c + aterm_offset(p, md.aterm_index, md.station2);

#ifdef _OPENMP
#pragma omp parallel for collapse(2)
#endif
        for (int y = 0; y < S; ++y) {
            for (int x = 0; x < S; ++x) {
                cf64 pix[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
                const double l = compute_l64(x, S, image_size);
                const double m = compute_l64(y, S, image_size);
                const double n = compute_n64(l, m);
                const double phase_offset = u_offset * l + v_offset * m + w_offset * n;
                for (int t = 0; t < md.nr_timesteps; ++t) {
                    const float *uvw_t = uvw + 3 * (size_t)(time_offset + t);
                    const double phase_index = (double)uvw_t[0] * l + (double)uvw_t[1] * m + (double)uvw_t[2] * n;
                    for (int c = 0; c < C; ++c) {
                        const double phase = phase_offset - phase_index * (double)wavenumbers[c];
                        const cf64 phasor = {cos(phase), sin(phase)};
                        const cf32 *v = vis_c + ((size_t)(time_offset + t) * C + c) * 4;
                        for (int pol = 0; pol < 4; ++pol) {
                            const cf64 vv = {v[pol].re, v[pol].im};
                            pix[pol] = cadd64(pix[pol], cmul64(vv, phasor));
                        }
                    }
                }
                const size_t px = ((size_t)y * S + x) * 4;
                cf64 A1[4], A2[4];
                for (int k = 0; k < 4; ++k) {
                    A1[k].re = a1[px + k].re; A1[k].im = a1[px + k].im;
                    A2[k].re = a2[px + k].re; A2[k].im = a2[px + k].im;
                }
                aterm_gridder64(pix, A1, A2);
                const double sph = spheroidal[y * S + x];
                for (int pol = 0; pol < 4; ++pol) {
                    cf64 *dst = sub_c + (((size_t)s * 4 + pol) * S + y) * S + x;
                    dst->re = pix[pol].re * sph;
                    dst->im = pix[pol].im * sph;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Degridder                                                          */
/* ------------------------------------------------------------------ */
void oracle_degridder_f32(const oracle_params *p, int aterm_mode, const float *uvw,
                          const float *wavenumbers, const float *subgrids, const float *spheroidal,
                          const float *aterms, const oracle_metadata *metadata, float *vis) {
    const int S = p->subgrid_size, C = p->nr_channels;
    const float image_size = p->image_size;
    const int baseline_offset_1 = metadata[0].baseline_offset;
    const cf32 *aterms_c = (const cf32 *)aterms;
    const cf32 *sub_c = (const cf32 *)subgrids;
    cf32 *vis_c = (cf32 *)vis;
    cf32 *pixels = (cf32 *)malloc(sizeof(cf32) * (size_t)S * S * 4);

    for (int s = 0; s < p->nr_subgrids; ++s) {
        const oracle_metadata md = metadata[s];
        const int time_offset = (md.baseline_offset - baseline_offset_1) + md.time_offset;
        const float w_offset_in_lambda = (float)((double)p->w_step * (md.z + 0.5));
        const cf32 *a1 = aterms_c + aterm_offset(p, md.aterm_index, md.station1);
        const cf32 *a2 = aterms_c + aterm_offset(p, md.aterm_index, md.station2);

#ifdef _OPENMP
#pragma omp parallel for collapse(2)
#endif
        for (int y = 0; y < S; ++y) {
            for (int x = 0; x < S; ++x) {
                const size_t px = ((size_t)y * S + x) * 4;
                const float sph = spheroidal[y * S + x];
                cf32 pix[4];
                for (int pol = 0; pol < 4; ++pol) {
                    const cf32 src = sub_c[(((size_t)s * 4 + pol) * S + y) * S + x];
                    pix[pol].re = sph * src.re;
                    pix[pol].im = sph * src.im;
                }
                if (aterm_mode == ORACLE_ATERM_ADJOINT)
                    aterm_degridder32(pix, a1 + px, a2 + px);
                else
                    aterm_gridder32(pix, a1 + px, a2 + px);
                for (int pol = 0; pol < 4; ++pol) pixels[px + pol] = pix[pol];
            }
        }

        /* degridding_benchmark.cpp:123-129: the offsets go through double */
        const float u_offset = (float)((double)((float)md.x + (float)S / 2 - (float)p->grid_size / 2) *
                                       (2 * M_PI / (double)image_size));
        const float v_offset = (float)((double)((float)md.y + (float)S / 2 - (float)p->grid_size / 2) *
                                       (2 * M_PI / (double)image_size));
        const float w_offset = (float)(2 * M_PI * (double)w_offset_in_lambda);

#ifdef _OPENMP
#pragma omp parallel for collapse(2)
#endif
        for (int t = 0; t < md.nr_timesteps; ++t) {
            for (int c = 0; c < C; ++c) {
                const float *uvw_t = uvw + 3 * (size_t)(time_offset + t);
                const float u = uvw_t[0], v = uvw_t[1], w = uvw_t[2];
                cf32 sum[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                for (int y = 0; y < S; ++y) {
                    for (int x = 0; x < S; ++x) {
                        const float l = compute_l32(x, S, image_size);
                        const float m = compute_l32(y, S, image_size);
                        const float n = compute_n32(l, m);
                        const float phase_index = u * l + v * m + w * n;
                        const float phase_offset = u_offset * l + v_offset * m + w_offset * n;
                        const float phase = (phase_index * wavenumbers[c]) - phase_offset;
                        const cf32 phasor = {cosf(phase), sinf(phase)};
                        const cf32 *pp = pixels + ((size_t)y * S + x) * 4;
                        for (int pol = 0; pol < 4; ++pol) sum[pol] = cadd32(sum[pol], cmul32(pp[pol], phasor));
                    }
                }
                cf32 *dst = vis_c + ((size_t)(time_offset + t) * C + c) * 4;
                for (int pol = 0; pol < 4; ++pol) dst[pol] = sum[pol];
            }
        }
    }
    free(pixels);
}

void oracle_degridder_f64(const oracle_params *p, int aterm_mode, const float *uvw,
                          const float *wavenumbers, const float *subgrids, const float *spheroidal,
                          const float *aterms, const oracle_metadata *metadata, double *vis) {
    const int S = p->subgrid_size, C = p->nr_channels;
    const double image_size = p->image_size;
    const int baseline_offset_1 = metadata[0].baseline_offset;
    const cf32 *aterms_c = (const cf32 *)aterms;
    const cf32 *sub_c = (const cf32 *)subgrids;
    cf64 *vis_c = (cf64 *)vis;
    cf64 *pixels = (cf64 *)malloc(sizeof(cf64) * (size_t)S * S * 4);
    double *lmn = (double *)malloc(sizeof(double) * (size_t)S * S * 3);

    for (int y = 0; y < S; ++y)
        for (int x = 0; x < S; ++x) {
            const double l = compute_l64(x, S, image_size), m = compute_l64(y, S, image_size);
            lmn[(y * S + x) * 3 + 0] = l;
            lmn[(y * S + x) * 3 + 1] = m;
            lmn[(y * S + x) * 3 + 2] = compute_n64(l, m);
        }

    for (int s = 0; s < p->nr_subgrids; ++s) {
        const oracle_metadata md = metadata[s];
        const int time_offset = (md.baseline_offset - baseline_offset_1) + md.time_offset;
        const cf32 *a1 = aterms_c + aterm_offset(p, md.aterm_index, md.station1);
        const cf32 *a2 = aterms_c + aterm_offset(p, md.aterm_index, md.station2);
        for (int y = 0; y < S; ++y) {
            for (int x = 0; x < S; ++x) {
                const size_t px = ((size_t)y * S + x) * 4;
                const double sph = spheroidal[y * S + x];
                cf64 pix[4], A1[4], A2[4];
                for (int pol = 0; pol < 4; ++pol) {
                    const cf32 src = sub_c[(((size_t)s * 4 + pol) * S + y) * S + x];
                    pix[pol].re = sph * src.re;
                    pix[pol].im = sph * src.im;
                    A1[pol].re = a1[px + pol].re; A1[pol].im = a1[px + pol].im;
                    A2[pol].re = a2[px + pol].re; A2[pol].im = a2[px + pol].im;
                }
                if (aterm_mode == ORACLE_ATERM_ADJOINT)
                    aterm_degridder64(pix, A1, A2);
                else
                    aterm_gridder64(pix, A1, A2);
                for (int pol = 0; pol < 4; ++pol) pixels[px + pol] = pix[pol];
            }
        }
        const double u_offset = ((double)md.x + S / 2.0 - p->grid_size / 2.0) * (2.0 * M_PI / image_size);
        const double v_offset = ((double)md.y + S / 2.0 - p->grid_size / 2.0) * (2.0 * M_PI / image_size);
        const double w_offset = 2.0 * M_PI * (double)p->w_step * (md.z + 0.5);

#ifdef _OPENMP
#pragma omp parallel for collapse(2)
#endif
        for (int t = 0; t < md.nr_timesteps; ++t) {
            for (int c = 0; c < C; ++c) {
                const float *uvw_t = uvw + 3 * (size_t)(time_offset + t);
                const double u = uvw_t[0], v = uvw_t[1], w = uvw_t[2];
                const double k = wavenumbers[c];
                cf64 sum[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
                for (int q = 0; q < S * S; ++q) {
                    const double l = lmn[q * 3], m = lmn[q * 3 + 1], n = lmn[q * 3 + 2];
                    const double phase = (u * l + v * m + w * n) * k - (u_offset * l + v_offset * m + w_offset * n);
                    const cf64 phasor = {cos(phase), sin(phase)};
                    for (int pol = 0; pol < 4; ++pol) sum[pol] = cadd64(sum[pol], cmul64(pixels[(size_t)q * 4 + pol], phasor));
                }
                cf64 *dst = vis_c + ((size_t)(time_offset + t) * C + c) * 4;
                for (int pol = 0; pol < 4; ++pol) dst[pol] = sum[pol];
            }
        }
    }
    free(lmn);
    free(pixels);
}

/* ------------------------------------------------------------------ */
/* Subgrid DFT (separable, FP64)                                      */
/* ------------------------------------------------------------------ */
void oracle_subgrid_dft_f64(int nr_subgrids, int S, int direction, const float *taper,
                            const double *in, double *out) {
    const double sgn = direction >= 0 ? 1.0 : -1.0;
    /* tw[o][i]: output index o, input index i.
     * forward : o = uv cell k, i = pixel x: e^{+2 pi i (k-S/2)(x-S/2+1/2)/S}
     * backward: o = pixel x, i = uv cell k: e^{-2 pi i (k-S/2)(x-S/2+1/2)/S} */
    cf64 *tw = (cf64 *)malloc(sizeof(cf64) * (size_t)S * S);
    for (int k = 0; k < S; ++k)
        for (int x = 0; x < S; ++x) {
            const double arg = sgn * 2.0 * M_PI * ((double)k - S / 2.0) * ((double)x - S / 2.0 + 0.5) / (double)S;
            const size_t idx = direction >= 0 ? (size_t)k * S + x : (size_t)x * S + k;
            tw[idx].re = cos(arg);
            tw[idx].im = sin(arg);
        }
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        cf64 *a = (cf64 *)malloc(sizeof(cf64) * (size_t)S * S);
        cf64 *b = (cf64 *)malloc(sizeof(cf64) * (size_t)S * S);
#ifdef _OPENMP
#pragma omp for
#endif
        for (int sp = 0; sp < nr_subgrids * 4; ++sp) {
            const cf64 *src = (const cf64 *)in + (size_t)sp * S * S;
            cf64 *dst = (cf64 *)out + (size_t)sp * S * S;
            for (int q = 0; q < S * S; ++q) {
                a[q] = src[q];
                if (direction >= 0 && taper) { a[q].re *= taper[q]; a[q].im *= taper[q]; }
            }
            /* transform along x: b[y][k] = sum_x a[y][x] tw[k][x] */
            for (int y = 0; y < S; ++y)
                for (int k = 0; k < S; ++k) {
                    cf64 acc = {0, 0};
                    for (int x = 0; x < S; ++x) acc = cadd64(acc, cmul64(a[y * S + x], tw[k * S + x]));
                    b[y * S + k] = acc;
                }
            /* transform along y: dst[j][k] = sum_y b[y][k] tw[j][y] */
            for (int j = 0; j < S; ++j)
                for (int k = 0; k < S; ++k) {
                    cf64 acc = {0, 0};
                    for (int y = 0; y < S; ++y) acc = cadd64(acc, cmul64(b[y * S + k], tw[j * S + y]));
                    dst[j * S + k] = acc;
                }
            if (direction < 0 && taper)
                for (int q = 0; q < S * S; ++q) { dst[q].re *= taper[q]; dst[q].im *= taper[q]; }
        }
        free(a);
        free(b);
    }
    free(tw);
}

/* ------------------------------------------------------------------ */
/* Adder / splitter                                                   */
/* ------------------------------------------------------------------ */
/* Grid cell of subgrid cell (j, i) of an entry: plane, polarisation, row,
 * column and the conjugation flag.  z in [0, W): direct.  z in [-W, 0): the
 * Hermitian mirror -- plane -z-1, cell (G - gy, G - gx), xy <-> yx, conjugate.
 * Returns 0 when the cell (or the entry's plane) is outside the grid. */
static int oracle_grid_cell(const oracle_metadata *md, int G, int W, int pol, int j, int i, long *plane, int *gpol,
                            long *gy, long *gx, int *conj) {
    if (md->z >= 0 && md->z < W) {
        *plane = md->z;
        *gpol = pol;
        *gy = (long)md->y + j;
        *gx = (long)md->x + i;
        *conj = 0;
    } else if (md->z < 0 && md->z >= -W) {
        *plane = -(long)md->z - 1;
        *gpol = (pol == 1 || pol == 2) ? 3 - pol : pol;
        *gy = (long)G - ((long)md->y + j);
        *gx = (long)G - ((long)md->x + i);
        *conj = 1;
    } else {
        return 0;
    }
    return *gy >= 0 && *gy < G && *gx >= 0 && *gx < G;
}

void oracle_adder_f64(int nr_subgrids, int S, int G, int W, const oracle_metadata *metadata,
                      const double *subgrids, double *grid) {
    for (int s = 0; s < nr_subgrids; ++s) {
        const oracle_metadata md = metadata[s];
        for (int pol = 0; pol < 4; ++pol)
            for (int j = 0; j < S; ++j)
                for (int i = 0; i < S; ++i) {
                    long plane, gy, gx;
                    int gpol, cj;
                    if (!oracle_grid_cell(&md, G, W, pol, j, i, &plane, &gpol, &gy, &gx, &cj)) continue;
                    const size_t src = ((((size_t)s * 4 + pol) * S + j) * S + i) * 2;
                    const size_t dst = (((((size_t)plane * 4 + gpol) * G) + gy) * G + gx) * 2;
                    grid[dst] += subgrids[src];
                    grid[dst + 1] += cj ? -subgrids[src + 1] : subgrids[src + 1];
                }
    }
}

void oracle_splitter_f64(int nr_subgrids, int S, int G, int W, const oracle_metadata *metadata,
                         const double *grid, double *subgrids) {
    for (int s = 0; s < nr_subgrids; ++s) {
        const oracle_metadata md = metadata[s];
        for (int pol = 0; pol < 4; ++pol)
            for (int j = 0; j < S; ++j)
                for (int i = 0; i < S; ++i) {
                    const size_t dst = ((((size_t)s * 4 + pol) * S + j) * S + i) * 2;
                    long plane, gy, gx;
                    int gpol, cj;
                    if (!oracle_grid_cell(&md, G, W, pol, j, i, &plane, &gpol, &gy, &gx, &cj)) {
                        subgrids[dst] = 0;
                        subgrids[dst + 1] = 0;
                        continue;
                    }
                    const size_t src = (((((size_t)plane * 4 + gpol) * G) + gy) * G + gx) * 2;
                    subgrids[dst] = grid[src];
                    subgrids[dst + 1] = cj ? -grid[src + 1] : grid[src + 1];
                }
    }
}

/* ------------------------------------------------------------------ */
/* Timed CPU baseline entry points                                    */
/* ------------------------------------------------------------------ */
int oracle_omp_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_cpu_gridding_omp(const oracle_params *p, const float *uvw, const float *wavenumbers,
                            const float *vis, const float *spheroidal, const float *aterms,
                            const oracle_metadata *metadata, float *subgrids) {
    oracle_gridder_f32(p, uvw, wavenumbers, vis, spheroidal, aterms, metadata, subgrids);
    return oracle_omp_max_threads();
}

int oracle_cpu_degridding_omp(const oracle_params *p, const float *uvw, const float *wavenumbers,
                              const float *subgrids, const float *spheroidal, const float *aterms,
                              const oracle_metadata *metadata, float *vis) {
    oracle_degridder_f32(p, ORACLE_ATERM_REFCPU, uvw, wavenumbers, subgrids, spheroidal, aterms, metadata, vis);
    return oracle_omp_max_threads();
}
