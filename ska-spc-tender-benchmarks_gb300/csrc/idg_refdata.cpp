// idg_refdata.cpp -- the reference benchmark's synthetic inputs, restated.
//
// Produces, value for value, what launch_gridding() fills before it dispatches
// (gridding/src/gridding_benchmark.cpp:203-213): srand(0) and then, in order,
// initialize_uvw, _frequencies, _wavenumbers, _visibilities, _baselines,
// _spheroidal, _aterms and _metadata (gridding/src/gridding_initialization.cpp:7-182).
// The float/double mix of every expression follows the reference's so the
// results are bitwise identical on glibc (same rand() sequence and libm on
// x86-64 and aarch64).  The plan this produces places subgrids at random grid
// coordinates (gridding_initialization.cpp:172-173); it is the reference's
// plan, not a uvw-driven one.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "../../include/idg_gb300.h"

namespace idg {

namespace {
inline float rand_normalized_float() { return static_cast<float>(rand()) / static_cast<float>(RAND_MAX); }
} // namespace

int reference_dataset(int64_t grid_size, int64_t S, int64_t nstations, int64_t C, int64_t ntimeslots, int64_t T,
                      float image_size, float *uvw, float *frequencies, float *wavenumbers, void *visibilities,
                      uint32_t *baselines, float *spheroidal, void *aterms, idg_metadata *metadata) {
    const int64_t nb = nstations * (nstations - 1) / 2;
    const int64_t nsg = nb * ntimeslots;
    const double speed_of_light = 299792458.0;

    srand(0);

    // initialize_uvw: one ellipse per subgrid row block (gridding_initialization.cpp:12-36)
    for (int64_t bl = 0; bl < nsg; ++bl) {
        const float half_grid_size = 0.5F * static_cast<float>((unsigned)grid_size);
        const float radius_u = half_grid_size + rand_normalized_float() * half_grid_size;
        const float radius_v = half_grid_size + rand_normalized_float() * half_grid_size;
        const float angle_step = 1.F / static_cast<float>(T);
        for (int64_t it = 0; it < T; ++it) {
            const float angle = (static_cast<float>(it) + 0.5) * angle_step;
            float *p = uvw + 3 * (bl * T + it);
            p[0] = radius_u * std::cos(angle * M_PI);
            p[1] = radius_v * std::sin(angle * M_PI);
            p[2] = 0;
        }
    }

    // initialize_frequencies / _wavenumbers (:38-60)
    std::vector<float> freq_local;
    float *freq = frequencies;
    if (!freq) {
        freq_local.resize((size_t)C);
        freq = freq_local.data();
    }
    {
        const size_t start_frequency = 150e6;
        const float frequency_increment = 0.7e6;
        for (size_t i = 0; i < (size_t)C; ++i) {
            const double frequency = start_frequency + frequency_increment * i;
            freq[i] = frequency;
        }
        for (size_t i = 0; i < (size_t)C; ++i) wavenumbers[i] = 2 * M_PI * freq[i] / speed_of_light;
    }

    // initialize_visibilities: a point source at (0.6 G, 0.7 G) cells (:62-94)
    {
        auto *vis = reinterpret_cast<std::complex<float> *>(visibilities);
        const float x_offset = 0.6 * (unsigned)grid_size;
        const float y_offset = 0.7 * (unsigned)grid_size;
        const float amplitude = 1.0f;
        const float l = x_offset * image_size / (unsigned)grid_size;
        const float m = y_offset * image_size / (unsigned)grid_size;
        for (int64_t bl = 0; bl < nsg; ++bl)
            for (int64_t t = 0; t < T; ++t)
                for (int64_t c = 0; c < C; ++c) {
                    const float *p = uvw + 3 * (bl * T + t);
                    const float u = (freq[c] / speed_of_light) * p[0];
                    const float v = (freq[c] / speed_of_light) * p[1];
                    const std::complex<float> value = amplitude * exp(std::complex<float>(0, -2 * M_PI * (u * l + v * m)));
                    std::complex<float> *dst = vis + ((bl * T + t) * C + c) * 4;
                    dst[0] = value * 1.01f;
                    dst[1] = value * 1.02f;
                    dst[2] = value * 1.03f;
                    dst[3] = value * 1.04f;
                }
    }

    // initialize_baselines (:96-113)
    std::vector<uint32_t> bl_local;
    uint32_t *bls = baselines;
    if (!bls) {
        bl_local.resize((size_t)nb * 2);
        bls = bl_local.data();
    }
    {
        unsigned bl = 0;
        for (unsigned s1 = 0; s1 < (unsigned)nstations; s1++)
            for (unsigned s2 = s1 + 1; s2 < (unsigned)nstations; s2++) {
                if (bl >= (unsigned)nb) break;
                bls[2 * bl] = s1;
                bls[2 * bl + 1] = s2;
                bl++;
            }
    }

    // initialize_spheroidal: a separable tent (:115-128)
    for (unsigned y = 0; y < (unsigned)S; y++) {
        const float tmp_y = std::fabs(-1 + y * 2.0f / float(S));
        for (unsigned x = 0; x < (unsigned)S; x++) {
            const float tmp_x = std::fabs(-1 + x * 2.0f / float(S));
            spheroidal[y * S + x] = tmp_y * tmp_x;
        }
    }

    // initialize_aterms (:130-156)
    {
        auto *at = reinterpret_cast<std::complex<float> *>(aterms);
        for (int64_t ts = 0; ts < ntimeslots; ts++)
            for (int64_t st = 0; st < nstations; st++)
                for (int64_t y = 0; y < S; y++)
                    for (int64_t x = 0; x < S; x++) {
                        const float scale = 0.8 + ((double)rand() / (double)(RAND_MAX) * 0.4);
                        const float value = spheroidal[y * S + x] * scale;
                        std::complex<float> *j = at + (((ts * nstations + st) * S + y) * S + x) * 4;
                        j[0] = std::complex<float>(value + 0.1, -0.1);
                        j[1] = std::complex<float>(value - 0.2, 0.1);
                        j[2] = std::complex<float>(value - 0.2, 0.1);
                        j[3] = std::complex<float>(value + 0.1, -0.1);
                    }
    }

    // initialize_metadata: random subgrid corners (:158-182)
    for (unsigned bl = 0; bl < (unsigned)nb; bl++)
        for (unsigned ts = 0; ts < (unsigned)ntimeslots; ts++) {
            idg_metadata md;
            md.baseline_offset = 0;
            md.time_offset = bl * (unsigned)ntimeslots * (unsigned)T + ts * (unsigned)T;
            md.nr_timesteps = (int)T;
            md.aterm_index = 0;
            md.station1 = bls[2 * bl];
            md.station2 = bls[2 * bl + 1];
            md.x = (double)rand() / (double)(RAND_MAX) * (unsigned)grid_size;
            md.y = (double)rand() / (double)(RAND_MAX) * (unsigned)grid_size;
            md.z = 0;
            metadata[bl * ntimeslots + ts] = md;
        }
    return 0;
}

} // namespace idg
