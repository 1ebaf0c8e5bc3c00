// nb_law.cuh -- the pairwise force law in FP32, shared by the direct-sum
// kernels (plain and batched).
//
// Reference law (Phys::Gravity, src/Sim/Physics.hpp:25-35, S = softening2):
//     a_i += m_j (p_j - p_i) / (r (r^2 + S)),   r = |p_j - p_i|
// with one MUFU.RSQ per pair: 1/(r (r^2+S)) = rsqrt(r^2 (r^2+S)^2 + tiny);
// tiny keeps the self pair's factor m rsqrt(tiny) finite, so that it adds
// exactly zero (times dp = 0).  tiny is 1e-30 unless the state's largest mass
// needs more (self_pair_tiny): masses above 1e21, as in the reference's own
// seeders (1e20..1e30), would make m * 1e15 overflow to inf and the self
// pair inf * 0 = NaN.  The raised tiny stays far below r^2 (r^2+S)^2 of any
// real pair at such scales.
// Plummer law: a_i += m_j (p_j - p_i) (r^2 + S)^{-3/2}.
#pragma once
#include "nb_common.cuh"
#include "../../include/nbody_gb300.h"

namespace nb {

constexpr int kFold = 32;            // sources summed in plain FP32 before a Kahan fold
constexpr float kTiny = 1e-30f;

// tiny for a state whose largest |mass| has the float bits *mmax_bits: the
// self pair's factor m / sqrt(tiny) stays <= 1e36 (1e-30 for masses <= 1e21).
__device__ __forceinline__ float self_pair_tiny(const unsigned* __restrict__ mmax_bits) {
    const float q = __uint_as_float(*mmax_bits) * 1e-36f;
    return fmaxf(kTiny, q * q);
}

template <int LAW>
__device__ __forceinline__ void interact(const float4 pj, float xi, float yi, float zi, float S, float tiny,
                                         float& ax, float& ay, float& az) {
    float dx = pj.x - xi;
    float dy = pj.y - yi;
    float dz = pj.z - zi;
    if (LAW == NB_LAW_REFERENCE) {
        float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        float s = r2 + S;
        float t = fmaf(r2 * s, s, tiny);
        float w = pj.w * rsqrt_approx(t);
        ax = fmaf(w, dx, ax);
        ay = fmaf(w, dy, ay);
        az = fmaf(w, dz, az);
    } else {
        float q = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, S)));
        float inv = rsqrt_approx(q);
        float w = pj.w * inv * (inv * inv);
        ax = fmaf(w, dx, ax);
        ay = fmaf(w, dy, ay);
        az = fmaf(w, dz, az);
    }
}

// The same interaction for two target bodies at once with the packed FP32x2
// instructions of sm_100+ (FADD2 / FMUL2 / FFMA2): identical operations in
// identical order, half the issue slots.  n* hold the negated target
// coordinates, so dx = xj + (-xi) rounds exactly like xj - xi.
template <int LAW>
__device__ __forceinline__ void interact_x2(float2 jx, float2 jy, float2 jz, float2 jm, float2 nx, float2 ny,
                                            float2 nz, float2 S2, float2 T2, float2& ax, float2& ay, float2& az) {
    const float2 dx = __fadd2_rn(jx, nx);
    const float2 dy = __fadd2_rn(jy, ny);
    const float2 dz = __fadd2_rn(jz, nz);
    float2 w;
    if (LAW == NB_LAW_REFERENCE) {
        float2 r2 = __fmul2_rn(dx, dx);
        r2 = __ffma2_rn(dy, dy, r2);
        r2 = __ffma2_rn(dz, dz, r2);
        const float2 s = __fadd2_rn(r2, S2);
        const float2 t = __ffma2_rn(__fmul2_rn(r2, s), s, T2);
        w = __fmul2_rn(jm, make_float2(rsqrt_approx(t.x), rsqrt_approx(t.y)));
    } else {
        float2 q = __ffma2_rn(dx, dx, S2);
        q = __ffma2_rn(dy, dy, q);
        q = __ffma2_rn(dz, dz, q);
        const float2 inv = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
        w = __fmul2_rn(__fmul2_rn(jm, inv), __fmul2_rn(inv, inv));
    }
    ax = __ffma2_rn(w, dx, ax);
    ay = __ffma2_rn(w, dy, ay);
    az = __ffma2_rn(w, dz, az);
}

}  // namespace nb
