// nb_io.cpp -- .nbody files and the reference's own particle seeders (host).
//
// .nbody (src/States/Simulation/SimulationState.cpp:229-277, 317-331): raw
// little-endian 104-byte Particle records, nothing else.  Reading
// re-centres the positions on the centre of mass computed in long double
// and rounded to float, as InitParticlesFromFile does.
//
// Seeders (src/Sim/IParticleSeeder.hpp:12-50): the distributions of
// RandomSeeder (src/Sim/RandomSeeder.cpp:12-40), GalaxySeeder
// (src/Sim/GalaxySeeder.cpp:43-144) and StarSystemSeeder
// (src/Sim/StarSystemSeeder.cpp:17-55), drawn from this library's Philox
// streams: std::default_random_engine is implementation-defined (MSVC and
// libstdc++ differ), so the reference's exact streams cannot be reproduced.
#include "nb_rng.hpp"
#include "../../include/nbody_gb300.h"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
// Phys constants (src/Sim/Physics.hpp:9-17)
constexpr double kAU = 1.15e12, kM = 1000.0, kStarSystemScale = 20 * kAU;

struct Rng {
    nb::BodyRng r;
    Rng(uint64_t seed, uint64_t body, uint32_t stream) : r(seed, body, stream) {}
    double uni(double a, double b) { return a + (b - a) * r.uniform(); }
    double normal(double mean, double sd) {
        const double u1 = r.uniform(), u2 = r.uniform();
        return mean + sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

void set_common(nb_particle& p, double vx, double vy, double vz, double mass, float r, float g, float b) {
    p.velocity[0] = vx; p.velocity[1] = vy; p.velocity[2] = vz;
    p.forces[0] = p.forces[1] = p.forces[2] = 0.0;
    p.mass = mass;
    p.colour[0] = r; p.colour[1] = g; p.colour[2] = b; p.colour[3] = 1.0f;
    std::memcpy(p.original_colour, p.colour, sizeof p.colour);
    p._pad = 0.f;
}

// RandomSeeder: uniform cube [-500, 500]^3 / scale, velocity 1e16 along the
// normalised position, mass U(1e20, 1e30), colour U(0.2, 1).
void seed_random(uint64_t seed, float scale, nb_particle* out, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        Rng r(seed, i, 11);
        nb_particle& p = out[i];
        for (int a = 0; a < 3; ++a) p.position[a] = (float)r.uni(-500.0, 500.0) / scale;
        const float len = std::sqrt(p.position[0] * p.position[0] + p.position[1] * p.position[1] +
                                    p.position[2] * p.position[2]);
        double nv[3] = {0, 0, 0};
        if (len > 0) for (int a = 0; a < 3; ++a) nv[a] = p.position[a] / len;
        const double mass = r.uni(1e20, 1e30);
        const float c0 = (float)r.uni(0.2, 1.0), c1 = (float)r.uni(0.2, 1.0), c2 = (float)r.uni(0.2, 1.0);
        set_common(p, nv[0] * 1e16, nv[1] * 1e16, nv[2] * 1e16, mass, c0, c1, c2);
    }
}

// StarSystemSeeder: a star of 1e30 at the origin; planets on the z axis at
// U(4, 7) AU * M / StarSystemScale with velocity (U(1, 5) AU*M, that / 20, 0),
// mass U(1e10, 1e26).
void seed_star_system(uint64_t seed, nb_particle* out, size_t n) {
    if (n == 0) return;
    std::memset(out[0].position, 0, sizeof out[0].position);
    set_common(out[0], 0, 0, 0, 1e30, 0.6f, 1.0f, 1.0f);
    for (size_t i = 1; i < n; ++i) {
        Rng r(seed, i, 12);
        nb_particle& p = out[i];
        p.position[0] = 0.f;
        p.position[1] = 0.f;
        p.position[2] = (float)(r.uni(4.0 * kAU * kM, 7.0 * kAU * kM) / kStarSystemScale);
        const double vx = r.uni(1 * kAU * kM, 5 * kAU * kM);
        const double vy = r.uni(1 * kAU * kM, 5 * kAU * kM) / 20.0;
        const double mass = r.uni(1e10, 1e26);
        const float c0 = (float)r.uni(0.0, 0.4), c1 = (float)r.uni(0.2, 1.0), c2 = (float)r.uni(0.2, 1.0);
        set_common(p, vx, vy, 0.0, mass, c0, c1, c2);
    }
}

// GalaxySeeder: two spiral arms holding 80% of the bodies (positions lerped
// across each arm segment, velocity along the arm), the rest uniform in a
// disk of radius 720 around the centre with tangential velocity; heights
// N(0, 16); a random yaw/pitch/roll orientation; mass U(1e28, 1e30) for the
// disk bodies and 1e20 for arm bodies.
void rotate(const double R[9], float v[3]) {
    const double x = v[0], y = v[1], z = v[2];
    v[0] = (float)(R[0] * x + R[1] * y + R[2] * z);
    v[1] = (float)(R[3] * x + R[4] * y + R[5] * z);
    v[2] = (float)(R[6] * x + R[7] * y + R[8] * z);
}

void seed_galaxy(uint64_t seed, float scale, nb_particle* out, size_t n) {
    Rng g(seed, 0, 13);
    const double yaw = g.uni(0, 2 * kPi), pitch = g.uni(0, 2 * kPi), roll = g.uni(0, 2 * kPi);
    // rotation = roll (z) then pitch (x) then yaw (y), applied to row vectors
    const double cy = std::cos(yaw), sy = std::sin(yaw), cp = std::cos(pitch), sp = std::sin(pitch);
    const double cr = std::cos(roll), sr = std::sin(roll);
    const double R[9] = {cr * cy + sr * sp * sy, -sr * cy + cr * sp * sy, cp * sy,
                         sr * cp, cr * cp, -sp,
                         -cr * sy + sr * sp * cy, sr * sy + cr * sp * cy, cp * cy};
    size_t k = 0;
    const float arm_frac = 0.8f;
    const int loops = (int)std::floor(6.0f / 0.1f);
    const double per_loop = std::floor((double)n * (arm_frac / 2) / loops);
    for (int arm = 0; arm < 2 && k < n; ++arm) {
        const double offset = arm == 0 ? 0.0 : 3.14;
        double angle = 0.0, radius = 2.0;
        for (int l = 0; l < loops && k < n; ++l, angle += 0.1, radius += 7.2) {
            const double sx0 = std::cos(angle + offset) * radius, sy0 = std::sin(angle + offset) * radius;
            const double nx0 = std::cos(angle + offset + 0.1) * (radius + 10.0);
            const double ny0 = std::sin(angle + offset + 0.1) * (radius + 10.0);
            double nmx = sx0 - nx0, nmy = sy0 - ny0;
            const double mag = std::sqrt(nmx * nmx + nmy * nmy);
            nmx /= mag; nmy /= mag;
            const double tx = nmy, ty = -nmx;   // normal x (0,0,1)
            for (int i = 0; i < (int)per_loop && k < n; ++i, ++k) {
                Rng r(seed, k, 14);
                const double a = r.normal(0.5, 0.2), b = r.uni(0.2, 0.5);
                float pos[3] = {(float)((sx0 - tx * 140) + a * 280 * tx + (sx0 - nmx * 400) + b * 800 * nmx),
                                (float)((sy0 - ty * 140) + a * 280 * ty + (sy0 - nmy * 400) + b * 800 * nmy),
                                (float)r.normal(0.0, 16.0)};
                const double vs = 2e16 * (1000.0 / mag);
                for (int q = 0; q < 3; ++q) pos[q] /= scale;
                rotate(R, pos);
                nb_particle& p = out[k];
                std::memcpy(p.position, pos, sizeof pos);
                set_common(p, nmx * vs, nmy * vs, 0.0, 1e20, (float)r.uni(0, 1), (float)r.uni(0, 1),
                           (float)r.uni(0, 1));
            }
        }
    }
    for (; k < n; ++k) {
        Rng r(seed, k, 15);
        float pos[3];
        do {
            pos[0] = (float)r.uni(-2000.0, 2000.0);
            pos[1] = (float)r.uni(-2000.0, 2000.0);
        } while ((double)pos[0] * pos[0] + (double)pos[1] * pos[1] > 720.0 * 720.0);
        pos[2] = (float)r.normal(0.0, 16.0);
        const double tx = pos[1], ty = -pos[0];   // (pos - centre) x (0,0,1)
        const double vs = r.uni(0.8, 1.2) * 1e14;
        for (int q = 0; q < 3; ++q) pos[q] /= scale;
        rotate(R, pos);
        nb_particle& p = out[k];
        std::memcpy(p.position, pos, sizeof pos);
        set_common(p, tx * vs, ty * vs, 0.0, r.uni(1e28, 1e30), (float)r.uni(0, 1), (float)r.uni(0, 1),
                   (float)r.uni(0, 1));
    }
}

}  // namespace

extern "C" {

int nb_seed_reference(int seeder, uint64_t seed, float scale, nb_particle* out, size_t n) {
    if ((!out && n) || !(scale > 0)) return NB_EINVAL;
    switch (seeder) {
        case 0: seed_random(seed, scale, out, n); return NB_OK;
        case 1: seed_galaxy(seed, scale, out, n); return NB_OK;
        case 2: seed_star_system(seed, out, n); return NB_OK;
        default: return NB_EINVAL;
    }
}

int nb_file_write(const char* path, const nb_particle* particles, size_t n) {
    if (!path || (!particles && n)) return NB_EINVAL;
    FILE* f = std::fopen(path, "wb");
    if (!f) return NB_EINVAL;
    const size_t w = n ? std::fwrite(particles, sizeof(nb_particle), n, f) : 0;
    const int rc = std::fclose(f);
    return (w == n && rc == 0) ? NB_OK : NB_EINVAL;
}

int nb_file_read(const char* path, nb_particle* particles, size_t capacity, size_t* n, int recentre) {
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
}

}  // extern "C"
