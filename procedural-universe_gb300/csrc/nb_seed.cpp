// nb_seed.cpp -- seeded initial conditions (host side).
//
// Synthetic galaxies for the workloads of the N-body step (Plummer spheres,
// exponential disk + Hernquist bulge galaxies, two Plummer spheres on a
// parabolic orbit), one body at a time from nb_seed_body.hpp, which the
// device generator of the batched and served forms (nb_gen.cu) shares.
// All systems are shifted to their centre-of-mass frame (sums in body order,
// double) before rounding to float; every body mass is a float value.
//
// The reference's own seeders (src/Sim/RandomSeeder.cpp:12-40,
// src/Sim/GalaxySeeder.cpp:43-144, src/Sim/StarSystemSeeder.cpp:17-55) are
// restated in nb_seed_reference (nb_io.cpp) with the same distributions; their random
// streams cannot match (std::default_random_engine is implementation-defined).
#include "nb_rng.hpp"
#include "nb_seed_body.hpp"
#include "../../include/nbody_gb300.h"
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>
#include <functional>

namespace {

using nb::BodyRng;
using namespace nb::seedbody;

void parallel_for(size_t n, const std::function<void(size_t, size_t)>& fn) {
    unsigned hc = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 65536 || hc == 1) { fn(0, n); return; }
    std::vector<std::thread> th;
    const size_t per = (n + hc - 1) / hc;
    for (unsigned t = 0; t < hc; ++t) {
        const size_t b = t * per, e = std::min(n, b + per);
        if (b < e) th.emplace_back(fn, b, e);
    }
    for (auto& x : th) x.join();
}

void finish(std::vector<double>& x, std::vector<double>& v, std::vector<float>& m, size_t n, float* pos_mass4,
            float* vel4) {
    double M = 0, cx[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
    for (size_t i = 0; i < n; ++i) {
        M += m[i];
        for (int k = 0; k < 3; ++k) { cx[k] += m[i] * x[3 * i + k]; cv[k] += m[i] * v[3 * i + k]; }
    }
    if (M > 0) for (int k = 0; k < 3; ++k) { cx[k] /= M; cv[k] /= M; }
    parallel_for(n, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            for (int k = 0; k < 3; ++k) {
                pos_mass4[4 * i + k] = (float)(x[3 * i + k] - cx[k]);
                vel4[4 * i + k] = (float)(v[3 * i + k] - cv[k]);
            }
            pos_mass4[4 * i + 3] = m[i];
            vel4[4 * i + 3] = 0.f;
        }
    });
}

}  // namespace

extern "C" {

int nb_seed_plummer(uint64_t seed, size_t n, double total_mass, double a, float* pos_mass4, float* vel4) {
    try {
        if ((!pos_mass4 || !vel4) && n) return NB_EINVAL;
        if (!(a > 0) || !(total_mass > 0)) return NB_EINVAL;
        std::vector<double> x(3 * n), v(3 * n);
        std::vector<float> m(n, (float)(total_mass / (double)n));
        parallel_for(n, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) {
                BodyRng r(seed, i, kStreamPlummer);
                plummer_body(r, total_mass, a, &x[3 * i], &v[3 * i]);
            }
        });
        finish(x, v, m, n, pos_mass4, vel4);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_seed_disk(uint64_t seed, size_t n, double total_mass, double rd, double z0, double bulge_frac, double ab,
                 double dispersion, float* pos_mass4, float* vel4) {
    try {
        if ((!pos_mass4 || !vel4) && n) return NB_EINVAL;
        if (!(rd > 0) || !(z0 > 0) || bulge_frac < 0 || bulge_frac >= 1 || !(total_mass > 0)) return NB_EINVAL;
        if (bulge_frac > 0 && !(ab > 0)) return NB_EINVAL;
        const DiskParams p = disk_params(n, total_mass, rd, z0, bulge_frac, ab, dispersion);
        std::vector<double> x(3 * n), v(3 * n);
        std::vector<float> m(n);
        parallel_for(n, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) {
                BodyRng r(seed, i, kStreamDisk);
                m[i] = disk_body(r, i, p, &x[3 * i], &v[3 * i]);
            }
        });
        finish(x, v, m, n, pos_mass4, vel4);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_seed_collision(uint64_t seed, size_t n, double a, double separation, double pericentre, float* pos_mass4,
                      float* vel4) {
    try {
        if ((!pos_mass4 || !vel4) && n) return NB_EINVAL;
        if (!(a > 0) || !(separation > 0) || pericentre < 0 || pericentre > separation || n < 2) return NB_EINVAL;
        const size_t h = n / 2;
        std::vector<double> x(3 * n), v(3 * n);
        std::vector<float> m(n);
        // each sphere has mass 1; relative parabolic orbit of total mass 2 (G = 1)
        const double Mt = 2.0;
        const double vrel = std::sqrt(2.0 * Mt / separation);
        const double vt = std::sqrt(2.0 * Mt * pericentre) / separation;
        const double vr = -std::sqrt(std::max(0.0, vrel * vrel - vt * vt));
        const double rel_v[3] = {vr, vt, 0.0};
        const double rel_x[3] = {separation, 0.0, 0.0};
        parallel_for(n, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) {
                const bool second = i >= h;
                const size_t cnt = second ? n - h : h;
                BodyRng r(seed, i, kStreamCollision);
                plummer_body(r, 1.0, a, &x[3 * i], &v[3 * i]);
                const double sgn = second ? 0.5 : -0.5;
                for (int k = 0; k < 3; ++k) { x[3 * i + k] += sgn * rel_x[k]; v[3 * i + k] += sgn * rel_v[k]; }
                m[i] = (float)(1.0 / (double)cnt);
            }
        });
        finish(x, v, m, n, pos_mass4, vel4);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

}  // extern "C"
