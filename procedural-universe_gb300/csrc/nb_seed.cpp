// nb_seed.cpp -- seeded initial conditions (host side).
//
// Synthetic galaxies for the workloads of the N-body step, drawn per body
// from counter-based Philox streams (nb_rng.hpp), so that a galaxy depends
// only on (seed, n) and generation parallelises over bodies:
//   * Plummer sphere: positions by inversion of the cumulative mass profile
//     (Aarseth, Henon, Wielen 1974) with the radius cut at mass fraction
//     0.999; isotropic speeds by von Neumann rejection on q^2 (1-q^2)^{7/2}.
//   * Exponential disk + Hernquist bulge: disk radii R = -rd ln(u1 u2)
//     (cut at 20 rd), sech^2 heights z = z0 atanh(2u-1) (cut at 10 z0),
//     circular speed from the enclosed disk + bulge mass (spherical
//     approximation) plus Gaussian dispersion; bulge radii
//     r = ab sqrt(u)/(1 - sqrt(u)) (cut at 100 ab) with Gaussian velocities of
//     the isotropic Hernquist (1990, eq. 10) dispersion of the bulge alone,
//     redrawn above 0.95 of the escape speed.
//   * Two Plummer spheres on a parabolic orbit (G = 1).
// All systems are shifted to their centre-of-mass frame before rounding to
// float; every body mass is a float value.
//
// The reference's own seeders (src/Sim/RandomSeeder.cpp:12-40,
// src/Sim/GalaxySeeder.cpp:43-144, src/Sim/StarSystemSeeder.cpp:17-55) are
// restated in nb_seed_reference (nb_io.cpp) with the same distributions; their random
// streams cannot match (std::default_random_engine is implementation-defined).
#include "nb_rng.hpp"
#include "../../include/nbody_gb300.h"
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>
#include <functional>

namespace {

using nb::BodyRng;
constexpr double kPi = 3.14159265358979323846;

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

void iso_dir(BodyRng& r, double len, double out[3]) {
    const double z = 1.0 - 2.0 * r.uniform();
    const double ph = 2.0 * kPi * r.uniform();
    const double s = std::sqrt(std::max(0.0, 1.0 - z * z));
    out[0] = len * s * std::cos(ph);
    out[1] = len * s * std::sin(ph);
    out[2] = len * z;
}

double normal(BodyRng& r) {
    const double u1 = r.uniform(), u2 = r.uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
}

// Plummer body (G = 1): position and velocity of total mass M, scale a.
void plummer_body(BodyRng& r, double M, double a, double x[3], double v[3]) {
    const double u = 0.999 * r.uniform();
    const double rad = a / std::sqrt(std::pow(u, -2.0 / 3.0) - 1.0);
    iso_dir(r, rad, x);
    double q = 0.0;
    for (int k = 0; k < 10000; ++k) {
        const double qq = r.uniform(), g = 0.1 * r.uniform();
        if (g < qq * qq * std::pow(1.0 - qq * qq, 3.5)) { q = qq; break; }
    }
    const double ve = std::sqrt(2.0 * M) * std::pow(rad * rad + a * a, -0.25);
    iso_dir(r, q * ve, v);
}

double hernquist_sigma2(double r, double M, double a) {
    const double x = r / a;
    const double t1 = 12.0 * r * std::pow(r + a, 3) / std::pow(a, 4) * std::log((r + a) / r);
    const double t2 = r / (r + a) * (25.0 + 52.0 * x + 42.0 * x * x + 12.0 * x * x * x);
    return std::max(0.0, M / (12.0 * a) * (t1 - t2));
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
                BodyRng r(seed, i, 1);
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
        const size_t nb = (size_t)std::llround(bulge_frac * (double)n);
        const size_t nd = n - nb;
        const double Md = total_mass * (1.0 - bulge_frac), Mb = total_mass * bulge_frac;
        std::vector<double> x(3 * n), v(3 * n);
        std::vector<float> m(n);
        const float md = nd ? (float)(Md / (double)nd) : 0.f, mb = nb ? (float)(Mb / (double)nb) : 0.f;
        parallel_for(n, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) {
                BodyRng r(seed, i, 2);
                double* xi = &x[3 * i];
                double* vi = &v[3 * i];
                if (i < nd) {
                    double R = 0;
                    for (int k = 0; k < 1000; ++k) {
                        R = -rd * std::log(r.uniform() * r.uniform());
                        if (R <= 20.0 * rd) break;
                    }
                    double z = 0;
                    for (int k = 0; k < 1000; ++k) {
                        z = z0 * std::atanh(2.0 * r.uniform() - 1.0);
                        if (std::fabs(z) <= 10.0 * z0) break;
                    }
                    const double ph = 2.0 * kPi * r.uniform();
                    xi[0] = R * std::cos(ph); xi[1] = R * std::sin(ph); xi[2] = z;
                    const double menc = Md * (1.0 - (1.0 + R / rd) * std::exp(-R / rd)) + Mb * R * R / ((R + ab) * (R + ab));
                    const double vc = R > 0 ? std::sqrt(menc / R) : 0.0;
                    vi[0] = -vc * std::sin(ph) + dispersion * vc * normal(r);
                    vi[1] = vc * std::cos(ph) + dispersion * vc * normal(r);
                    vi[2] = dispersion * vc * normal(r);
                    m[i] = md;
                } else {
                    double rad = 0;
                    const double umax = (100.0 / 101.0) * (100.0 / 101.0);
                    for (int k = 0; k < 1000; ++k) {
                        const double u = r.uniform();
                        if (u > umax) continue;
                        const double s = std::sqrt(u);
                        rad = ab * s / (1.0 - s);
                        break;
                    }
                    iso_dir(r, rad, xi);
                    const double sig = std::sqrt(hernquist_sigma2(std::max(rad, 1e-12), Mb, ab));
                    const double vesc2 = 2.0 * Mb / (rad + ab);
                    for (int k = 0; k < 1000; ++k) {
                        vi[0] = sig * normal(r); vi[1] = sig * normal(r); vi[2] = sig * normal(r);
                        if (vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2] < 0.9025 * vesc2) break;
                    }
                    m[i] = mb;
                }
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
                BodyRng r(seed, i, 3);
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
