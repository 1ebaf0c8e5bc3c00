// nb_seed_body.hpp -- one body of the synthetic workload galaxies, shared by
// the host generator (nb_seed_*, nb_seed.cpp) and the device generator of the
// batched and served forms (nb_gen.cu).
//
// Every body draws from its own counter-based Philox stream (nb_rng.hpp), so
// a body depends only on (seed, index) and any thread on any device can make
// it.  The arithmetic is written once for both sides; on the device the
// double-precision math functions (log, exp, pow, sin, cos, atanh) are CUDA's
// and nvcc may contract multiply-adds, so a device body differs from the host
// body by the rounding of those operations (a few ulp in double).
//   * Plummer sphere (G = 1): radius by inversion of the cumulative mass
//     profile (Aarseth, Henon, Wielen 1974) cut at mass fraction 0.999;
//     isotropic speed by von Neumann rejection on q^2 (1 - q^2)^{7/2}.
//   * Exponential disk + Hernquist bulge: disk radii R = -rd ln(u1 u2) (cut
//     at 20 rd), sech^2 heights z = z0 atanh(2u - 1) (cut at 10 z0), circular
//     speed from the enclosed disk + bulge mass (spherical approximation) plus
//     Gaussian dispersion; bulge radii r = ab sqrt(u) / (1 - sqrt(u)) (cut at
//     100 ab) with Gaussian velocities of the isotropic Hernquist (1990,
//     eq. 10) dispersion of the bulge alone, redrawn above 0.95 of the escape
//     speed.
//   * Two Plummer spheres on a parabolic orbit.
// The centre-of-mass shift and the rounding to float follow in the callers.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>

#include "nb_rng.hpp"

namespace nb {
namespace seedbody {

constexpr double kPi = 3.14159265358979323846;

NB_HD double dmax(double a, double b) { return (a < b) ? b : a; }

NB_HD void iso_dir(BodyRng& r, double len, double out[3]) {
    const double z = 1.0 - 2.0 * r.uniform();
    const double ph = 2.0 * kPi * r.uniform();
    const double s = sqrt(dmax(0.0, 1.0 - z * z));
    out[0] = len * s * cos(ph);
    out[1] = len * s * sin(ph);
    out[2] = len * z;
}

NB_HD double normal(BodyRng& r) {
    const double u1 = r.uniform(), u2 = r.uniform();
    return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
}

// Plummer body (G = 1): position and velocity of total mass M, scale a.
NB_HD void plummer_body(BodyRng& r, double M, double a, double x[3], double v[3]) {
    const double u = 0.999 * r.uniform();
    const double rad = a / sqrt(pow(u, -2.0 / 3.0) - 1.0);
    iso_dir(r, rad, x);
    double q = 0.0;
    for (int k = 0; k < 10000; ++k) {
        const double qq = r.uniform(), g = 0.1 * r.uniform();
        if (g < qq * qq * pow(1.0 - qq * qq, 3.5)) { q = qq; break; }
    }
    const double ve = sqrt(2.0 * M) * pow(rad * rad + a * a, -0.25);
    iso_dir(r, q * ve, v);
}

NB_HD double hernquist_sigma2(double r, double M, double a) {
    const double x = r / a;
    const double t1 = 12.0 * r * pow(r + a, 3.0) / pow(a, 4.0) * log((r + a) / r);
    const double t2 = r / (r + a) * (25.0 + 52.0 * x + 42.0 * x * x + 12.0 * x * x * x);
    return dmax(0.0, M / (12.0 * a) * (t1 - t2));
}

// Parameters of a disk + bulge galaxy of n bodies: the first nd bodies are
// the disk, the rest the bulge.
struct DiskParams {
    double rd, z0, ab, dispersion, Md, Mb;
    size_t nd;
    float md, mb;
};

NB_HD DiskParams disk_params(size_t n, double total_mass, double rd, double z0, double bulge_frac, double ab,
                             double dispersion) {
    DiskParams p;
    const size_t nb = (size_t)llround(bulge_frac * (double)n);
    p.nd = n - nb;
    p.Md = total_mass * (1.0 - bulge_frac);
    p.Mb = total_mass * bulge_frac;
    p.md = p.nd ? (float)(p.Md / (double)p.nd) : 0.f;
    p.mb = nb ? (float)(p.Mb / (double)nb) : 0.f;
    p.rd = rd; p.z0 = z0; p.ab = ab; p.dispersion = dispersion;
    return p;
}

// Body i of a disk + bulge galaxy; returns its mass.
NB_HD float disk_body(BodyRng& r, size_t i, const DiskParams& p, double xi[3], double vi[3]) {
    if (i < p.nd) {
        double R = 0;
        for (int k = 0; k < 1000; ++k) {
            R = -p.rd * log(r.uniform() * r.uniform());
            if (R <= 20.0 * p.rd) break;
        }
        double z = 0;
        for (int k = 0; k < 1000; ++k) {
            z = p.z0 * atanh(2.0 * r.uniform() - 1.0);
            if (fabs(z) <= 10.0 * p.z0) break;
        }
        const double ph = 2.0 * kPi * r.uniform();
        xi[0] = R * cos(ph); xi[1] = R * sin(ph); xi[2] = z;
        const double menc = p.Md * (1.0 - (1.0 + R / p.rd) * exp(-R / p.rd)) + p.Mb * R * R / ((R + p.ab) * (R + p.ab));
        const double vc = R > 0 ? sqrt(menc / R) : 0.0;
        vi[0] = -vc * sin(ph) + p.dispersion * vc * normal(r);
        vi[1] = vc * cos(ph) + p.dispersion * vc * normal(r);
        vi[2] = p.dispersion * vc * normal(r);
        return p.md;
    }
    double rad = 0;
    const double umax = (100.0 / 101.0) * (100.0 / 101.0);
    for (int k = 0; k < 1000; ++k) {
        const double u = r.uniform();
        if (u > umax) continue;
        const double s = sqrt(u);
        rad = p.ab * s / (1.0 - s);
        break;
    }
    iso_dir(r, rad, xi);
    const double sig = sqrt(hernquist_sigma2(dmax(rad, 1e-12), p.Mb, p.ab));
    const double vesc2 = 2.0 * p.Mb / (rad + p.ab);
    for (int k = 0; k < 1000; ++k) {
        vi[0] = sig * normal(r); vi[1] = sig * normal(r); vi[2] = sig * normal(r);
        if (vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2] < 0.9025 * vesc2) break;
    }
    return p.mb;
}

// Streams of the three models (the third argument of BodyRng).
constexpr uint32_t kStreamPlummer = 1, kStreamDisk = 2, kStreamCollision = 3;

}  // namespace seedbody
}  // namespace nb
