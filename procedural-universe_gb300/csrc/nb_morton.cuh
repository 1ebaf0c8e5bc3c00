// nb_morton.cuh -- keys of the batched form's forest (shared by nb_tree.cu,
// which computes them together with the radix sort's histograms, and
// nb_batch_kernels.cuh, which bounds each galaxy).
//
// A Barnes-Hut member's key is its galaxy slot (21 bits, the top 7 octal
// levels) followed by a 42-bit Morton code of its position in the galaxy's
// bounding cube (14 levels).  The cube comes from per-galaxy min/max words
// kept as an order-preserving integer image of the floats.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nb {

constexpr int kSlotLevels = 7;          // 21 bits of galaxy slot
constexpr int kMortonLevels = 14;       // 42 bits of position in the galaxy cube
constexpr int kBatchDepth = kSlotLevels + kMortonLevels;

// Total order of floats as unsigned integers: -inf < ... < -0 < +0 < ... < +inf.
__device__ __forceinline__ unsigned float_to_ordered(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(unsigned o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// Galaxy g's cube (x0, y0, z0, edge) from its six ordered min/max words:
// the box's largest extent, widened by 0.1% so that the maximum maps inside.
__device__ __forceinline__ float4 gal_cube(const unsigned* __restrict__ bits, int g) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = ordered_to_float(bits[6 * g + a]);
        hi[a] = ordered_to_float(bits[6 * g + 3 + a]);
    }
    float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    ext = fmaxf(ext * 1.001f, 1e-20f);
    return make_float4(lo[0], lo[1], lo[2], ext);
}

__device__ __forceinline__ uint64_t spread3(uint32_t v) {   // 14 bits -> every third bit
    uint64_t x = v & 0x3fffu;
    x = (x | (x << 16)) & 0x0000ff0000ffull;
    x = (x | (x << 8)) & 0x00f00f00f00full;
    x = (x | (x << 4)) & 0x0c30c30c30c3ull;
    x = (x | (x << 2)) & 0x249249249249ull;
    return x;
}

__device__ __forceinline__ uint64_t forest_key(const float4 p, int slot, const float4 b) {
    const float sc = 16384.0f / b.w;
    const uint32_t qx = (uint32_t)fminf(fmaxf((p.x - b.x) * sc, 0.f), 16383.f);
    const uint32_t qy = (uint32_t)fminf(fmaxf((p.y - b.y) * sc, 0.f), 16383.f);
    const uint32_t qz = (uint32_t)fminf(fmaxf((p.z - b.z) * sc, 0.f), 16383.f);
    return ((uint64_t)slot << (3 * kMortonLevels)) | spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
}

}  // namespace nb
