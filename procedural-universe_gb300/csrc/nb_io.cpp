// nb_io.cpp -- .nbody files and the reference's own particle seeders (host).
//
// .nbody (src/States/Simulation/SimulationState.cpp:229-277, 317-331): raw
// little-endian 104-byte Particle records, nothing else.  Reading
// re-centres the positions on the centre of mass computed in long double
// and rounded to float, as InitParticlesFromFile does.
//
// Seeders: RandomSeeder, GalaxySeeder and StarSystemSeeder restated per body
// in nb_refseed.hpp (the GPU path, nb_init_seeded, runs the same functions).
#include "nb_refseed.hpp"
#include "../../include/nbody_gb300.h"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

extern "C" {

int nb_seed_reference(int seeder, uint64_t seed, float scale, nb_particle* out, size_t n) {
    try {
        if ((!out && n) || !(scale > 0)) return NB_EINVAL;
        namespace rs = nb::refseed;
        switch (seeder) {
            case 0:
                for (size_t i = 0; i < n; ++i) rs::random_body(seed, i, scale, out[i]);
                return NB_OK;
            case 1: {
                const rs::GalaxyFrame f = rs::galaxy_frame(seed, n);
                for (size_t i = 0; i < n; ++i) rs::galaxy_body(seed, i, scale, f, out[i]);
                return NB_OK;
            }
            case 2:
                for (size_t i = 0; i < n; ++i) rs::star_system_body(seed, i, out[i]);
                return NB_OK;
            default: return NB_EINVAL;
        }
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_file_write(const char* path, const nb_particle* particles, size_t n) {
    try {
        if (!path || (!particles && n)) return NB_EINVAL;
        FILE* f = std::fopen(path, "wb");
        if (!f) return NB_EINVAL;
        const size_t w = n ? std::fwrite(particles, sizeof(nb_particle), n, f) : 0;
        const int rc = std::fclose(f);
        return (w == n && rc == 0) ? NB_OK : NB_EINVAL;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_file_read(const char* path, nb_particle* particles, size_t capacity, size_t* n, int recentre) {
    try {
        if (!path || !n) return NB_EINVAL;
        FILE* f = std::fopen(path, "rb");
        if (!f) return NB_EINVAL;
        std::fseek(f, 0, SEEK_END);
        const long bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        // a trailing partial record is ignored, as the reference's read loop stops on it
        const size_t count = bytes > 0 ? (size_t)bytes / sizeof(nb_particle) : 0;
        *n = count;
        if (!particles) {
            std::fclose(f);
            return NB_OK;
        }
        if (capacity < count) {
            std::fclose(f);
            return NB_EINVAL;
        }
        const size_t got = count ? std::fread(particles, sizeof(nb_particle), count, f) : 0;
        std::fclose(f);
        if (got != count) return NB_EINVAL;
        if (recentre && count) {
            // TotalMass is a long double, CentreOfMass a double vector (SimulationState.cpp:250-264)
            long double M = 0.0L;
            double c[3] = {0.0, 0.0, 0.0};
            for (size_t i = 0; i < count; ++i) {
                M += particles[i].mass;
                for (int a = 0; a < 3; ++a) c[a] += (double)particles[i].position[a] * particles[i].mass;
            }
            if (M != 0.0L) {
                const double md = (double)M;
                const float centre[3] = {(float)(c[0] / md), (float)(c[1] / md), (float)(c[2] / md)};
                for (size_t i = 0; i < count; ++i)
                    for (int a = 0; a < 3; ++a) particles[i].position[a] = particles[i].position[a] - centre[a];
            }
        }
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

}  // extern "C"
