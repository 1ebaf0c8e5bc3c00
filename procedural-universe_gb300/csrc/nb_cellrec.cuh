// nb_cellrec.cuh -- the batched form's per-cell record (written by the
// topology's placement and the bottom-up moment pass, read by the traversal).
//
// One 64-byte record per cell, two 32-byte sectors:
//   sector 0: centre of mass and mass; the walk record
//             (first child or, for a leaf, first body; bodies; first body;
//              kind | children << 4 | level << 8)
//   sector 1: the traceless quadrupole Q_ij = sum m (3 y_i y_j - |y|^2 d_ij),
//             y = offset from the cell's centre of mass: (xx, yy, zz, 0),
//             (xy, xz, yz, 0)
// A walk step tests a child with one sector; only an accepted cell reads the
// second.  Each record is written whole by one thread (full sectors, no
// partial-sector write-back).
#pragma once
#include <cstdint>

namespace nb {

struct alignas(64) CellRec {
    float4 com;
    int4 walk;
    float4 q1;
    float4 q2;
};
static_assert(sizeof(CellRec) == 64, "two sectors per cell");

enum : int { BK_SINGLE = 1, BK_BUCKET = 2, BK_INTERNAL = 3 };

__device__ __forceinline__ int4 walk_record(int F, int count, int first, int kind, int nch, int level) {
    return make_int4(F, count, first, kind | (nch << 4) | (level << 8));
}

// Mass, centre of mass and quadrupole of the bodies [first, first + count)
// (two passes: centre of mass, then the moments about it).
__device__ __forceinline__ void bucket_moments(const float4* spos, int first, int count, float4& cm, float4& q1,
                                               float4& q2) {
    float m = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    for (int q = first; q < first + count; ++q) {
        const float4 b = spos[q];
        m += b.w; cx = fmaf(b.w, b.x, cx); cy = fmaf(b.w, b.y, cy); cz = fmaf(b.w, b.z, cz);
    }
    const float im = m > 0.f ? 1.f / m : 0.f;
    cx *= im; cy *= im; cz *= im;
    float xx = 0.f, yy = 0.f, zz = 0.f, xy = 0.f, xz = 0.f, yz = 0.f;
    for (int q = first; q < first + count; ++q) {
        const float4 b = spos[q];
        const float dx = b.x - cx, dy = b.y - cy, dz = b.z - cz, r2 = dx * dx + dy * dy + dz * dz;
        xx += b.w * (3.f * dx * dx - r2); yy += b.w * (3.f * dy * dy - r2); zz += b.w * (3.f * dz * dz - r2);
        xy += b.w * 3.f * dx * dy; xz += b.w * 3.f * dx * dz; yz += b.w * 3.f * dy * dz;
    }
    cm = make_float4(cx, cy, cz, m);
    q1 = make_float4(xx, yy, zz, 0.f);
    q2 = make_float4(xy, xz, yz, 0.f);
}

// A leaf's record: a single body (its position and mass, no quadrupole) or a
// depth-cap bucket of `count` bodies starting at sorted position s.
__device__ __forceinline__ void write_leaf_record(CellRec* rec, const float4* spos, int s, int count, int level) {
    float4 cm, q1 = make_float4(0.f, 0.f, 0.f, 0.f), q2 = q1;
    int kind = BK_SINGLE;
    if (count == 1) {
        cm = spos[s];
    } else {
        bucket_moments(spos, s, count, cm, q1, q2);
        kind = BK_BUCKET;
    }
    __stcg(&rec->com, cm);
    __stcg(&rec->walk, walk_record(s, count, s, kind, 0, level));
    __stcg(&rec->q1, q1);
    __stcg(&rec->q2, q2);
}

}  // namespace nb
