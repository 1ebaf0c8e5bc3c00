// nb_refseed.hpp -- the reference's particle seeders, one body at a time,
// shared by the host loop (nb_seed_reference, nb_io.cpp) and the GPU kernel
// (nb_init_seeded, nb_seed_gpu.cu).
//
// Distributions of RandomSeeder (src/Sim/RandomSeeder.cpp:12-40), GalaxySeeder
// (src/Sim/GalaxySeeder.cpp:43-144) and StarSystemSeeder
// (src/Sim/StarSystemSeeder.cpp:17-55), drawn from per-body Philox streams
// (nb_rng.hpp): std::default_random_engine is implementation-defined (MSVC and
// libstdc++ differ), so the reference's exact streams cannot be reproduced.
// Every body depends only on (seed, index), so any thread on any device
// generates it.
#pragma once
#include <cmath>
#include <cstring>

#include "../../include/nbody_gb300.h"
#include "nb_rng.hpp"

namespace nb {
namespace refseed {

constexpr double kPi = 3.14159265358979323846;
// Phys constants (src/Sim/Physics.hpp:9-17)
constexpr double kAU = 1.15e12, kM = 1000.0, kStarSystemScale = 20 * kAU;
constexpr int kGalaxyLoops = 60;        // floor(6.0f / 0.1f): spiral loops per arm
constexpr int kRejectCap = 4096;        // bound on the disk rejection loop (acceptance ~10%)

struct Rng {
    BodyRng r;
    NB_HD Rng(uint64_t seed, uint64_t body, uint32_t stream) : r(seed, body, stream) {}
    // a + (b - a) u, rounded the same way on host and device (no fused multiply-add)
    NB_HD double uni(double a, double b) {
#if defined(__CUDA_ARCH__)
        return __dadd_rn(a, __dmul_rn(b - a, r.uniform()));
#else
        return a + (b - a) * r.uniform();
#endif
    }
    NB_HD double normal(double mean, double sd) {
        const double u1 = r.uniform(), u2 = r.uniform();
        return mean + sd * sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
    }
};

NB_HD void set_common(nb_particle& p, double vx, double vy, double vz, double mass, float r, float g, float b) {
    p.velocity[0] = vx; p.velocity[1] = vy; p.velocity[2] = vz;
    p.forces[0] = p.forces[1] = p.forces[2] = 0.0;
    p.mass = mass;
    p.colour[0] = r; p.colour[1] = g; p.colour[2] = b; p.colour[3] = 1.0f;
    for (int k = 0; k < 4; ++k) p.original_colour[k] = p.colour[k];
    p._pad = 0.f;
}

// RandomSeeder: uniform cube [-500, 500]^3 / scale, velocity 1e16 along the
// normalised position, mass U(1e20, 1e30), colour U(0.2, 1).
NB_HD void random_body(uint64_t seed, size_t i, float scale, nb_particle& p) {
    Rng r(seed, i, 11);
    for (int a = 0; a < 3; ++a) p.position[a] = (float)r.uni(-500.0, 500.0) / scale;
    const float len = sqrtf(p.position[0] * p.position[0] + p.position[1] * p.position[1] +
                            p.position[2] * p.position[2]);
    double nv[3] = {0, 0, 0};
    if (len > 0) for (int a = 0; a < 3; ++a) nv[a] = p.position[a] / len;
    const double mass = r.uni(1e20, 1e30);
    const float c0 = (float)r.uni(0.2, 1.0), c1 = (float)r.uni(0.2, 1.0), c2 = (float)r.uni(0.2, 1.0);
    set_common(p, nv[0] * 1e16, nv[1] * 1e16, nv[2] * 1e16, mass, c0, c1, c2);
}

// StarSystemSeeder: a star of 1e30 at the origin; planets on the z axis at
// U(4, 7) AU * M / StarSystemScale with velocity (U(1, 5) AU*M, that / 20, 0),
// mass U(1e10, 1e26).
NB_HD void star_system_body(uint64_t seed, size_t i, nb_particle& p) {
    if (i == 0) {
        p.position[0] = p.position[1] = p.position[2] = 0.f;
        set_common(p, 0, 0, 0, 1e30, 0.6f, 1.0f, 1.0f);
        return;
    }
    Rng r(seed, i, 12);
    p.position[0] = 0.f;
    p.position[1] = 0.f;
    p.position[2] = (float)(r.uni(4.0 * kAU * kM, 7.0 * kAU * kM) / kStarSystemScale);
    const double vx = r.uni(1 * kAU * kM, 5 * kAU * kM);
    const double vy = r.uni(1 * kAU * kM, 5 * kAU * kM) / 20.0;
    const double mass = r.uni(1e10, 1e26);
    const float c0 = (float)r.uni(0.0, 0.4), c1 = (float)r.uni(0.2, 1.0), c2 = (float)r.uni(0.2, 1.0);
    set_common(p, vx, vy, 0.0, mass, c0, c1, c2);
}

// GalaxySeeder: two spiral arms holding 80% of the bodies (positions lerped
// across each arm segment, velocity along the arm), the rest uniform in a
// disk of radius 720 around the centre with tangential velocity; heights
// N(0, 16); one random yaw/pitch/roll orientation for the whole galaxy; mass
// U(1e28, 1e30) for the disk bodies and 1e20 for arm bodies.
struct GalaxyFrame {
    double R[9];        // rotation: roll (z), then pitch (x), then yaw (y), on row vectors
    long long per_loop; // bodies per arm segment
};

inline GalaxyFrame galaxy_frame(uint64_t seed, size_t n) {
    Rng g(seed, 0, 13);
    const double yaw = g.uni(0, 2 * kPi), pitch = g.uni(0, 2 * kPi), roll = g.uni(0, 2 * kPi);
    const double cy = std::cos(yaw), sy = std::sin(yaw), cp = std::cos(pitch), sp = std::sin(pitch);
    const double cr = std::cos(roll), sr = std::sin(roll);
    GalaxyFrame f;
    const double R[9] = {cr * cy + sr * sp * sy, -sr * cy + cr * sp * sy, cp * sy,
                         sr * cp, cr * cp, -sp,
                         -cr * sy + sr * sp * cy, sr * sy + cr * sp * cy, cp * cy};
    for (int k = 0; k < 9; ++k) f.R[k] = R[k];
    const float arm_frac = 0.8f;
    f.per_loop = (long long)std::floor((double)n * (arm_frac / 2) / kGalaxyLoops);
    return f;
}

NB_HD void rotate(const double R[9], float v[3]) {
    const double x = v[0], y = v[1], z = v[2];
    v[0] = (float)(R[0] * x + R[1] * y + R[2] * z);
    v[1] = (float)(R[3] * x + R[4] * y + R[5] * z);
    v[2] = (float)(R[6] * x + R[7] * y + R[8] * z);
}

NB_HD void galaxy_body(uint64_t seed, size_t k, float scale, const GalaxyFrame& f, nb_particle& p) {
    const long long arm_bodies = (long long)kGalaxyLoops * f.per_loop;
    if ((long long)k < 2 * arm_bodies) {
        const int arm = (int)((long long)k / arm_bodies);
        const int l = (int)(((long long)k % arm_bodies) / f.per_loop);
        const double offset = arm == 0 ? 0.0 : 3.14;
        const double angle = 0.1 * l, radius = 2.0 + 7.2 * l;
        const double sx0 = cos(angle + offset) * radius, sy0 = sin(angle + offset) * radius;
        const double nx0 = cos(angle + offset + 0.1) * (radius + 10.0);
        const double ny0 = sin(angle + offset + 0.1) * (radius + 10.0);
        double nmx = sx0 - nx0, nmy = sy0 - ny0;
        const double mag = sqrt(nmx * nmx + nmy * nmy);
        nmx /= mag;
        nmy /= mag;
        const double tx = nmy, ty = -nmx;   // normal x (0,0,1)
        Rng r(seed, k, 14);
        const double a = r.normal(0.5, 0.2), b = r.uni(0.2, 0.5);
        float pos[3] = {(float)((sx0 - tx * 140) + a * 280 * tx + (sx0 - nmx * 400) + b * 800 * nmx),
                        (float)((sy0 - ty * 140) + a * 280 * ty + (sy0 - nmy * 400) + b * 800 * nmy),
                        (float)r.normal(0.0, 16.0)};
        const double vs = 2e16 * (1000.0 / mag);
        for (int q = 0; q < 3; ++q) pos[q] /= scale;
        rotate(f.R, pos);
        for (int q = 0; q < 3; ++q) p.position[q] = pos[q];
        const float c0 = (float)r.uni(0, 1), c1 = (float)r.uni(0, 1), c2 = (float)r.uni(0, 1);
        set_common(p, nmx * vs, nmy * vs, 0.0, 1e20, c0, c1, c2);
        return;
    }
    Rng r(seed, k, 15);
    float pos[3] = {0.f, 0.f, 0.f};
    for (int it = 0; it < kRejectCap; ++it) {
        pos[0] = (float)r.uni(-2000.0, 2000.0);
        pos[1] = (float)r.uni(-2000.0, 2000.0);
        if ((double)pos[0] * pos[0] + (double)pos[1] * pos[1] <= 720.0 * 720.0) break;
        pos[0] = pos[1] = 0.f;   // (only kept if every draw is rejected)
    }
    pos[2] = (float)r.normal(0.0, 16.0);
    const double tx = pos[1], ty = -pos[0];   // (pos - centre) x (0,0,1)
    const double vs = r.uni(0.8, 1.2) * 1e14;
    for (int q = 0; q < 3; ++q) pos[q] /= scale;
    rotate(f.R, pos);
    for (int q = 0; q < 3; ++q) p.position[q] = pos[q];
    const double mass = r.uni(1e28, 1e30);
    const float c0 = (float)r.uni(0, 1), c1 = (float)r.uni(0, 1), c2 = (float)r.uni(0, 1);
    set_common(p, tx * vs, ty * vs, 0.0, mass, c0, c1, c2);
}

}  // namespace refseed
}  // namespace nb
