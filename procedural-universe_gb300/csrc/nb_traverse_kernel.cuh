// nb_traverse_kernel.cuh -- the K6 traversal kernel (included by nb_traverse.cu).
//
// Two bodies per lane: a warp walks for 64 consecutive bodies of the key
// order (lane l holds bodies base + l and base + 32 + l), so each popped cell
// and each loaded child serves twice as many bodies, and the arithmetic of
// both bodies runs in the packed FP32x2 instructions.  Every decision is
// still made per body exactly as the reference's recursion makes it: a stack
// entry carries one lane mask per body slot, the distance test uses the
// float operations of the reference (each element of a packed operation is
// rounded like its scalar counterpart), and a body whose test does not
// accept contributes zero through a zero mass in the packed interaction.
// Only the rare cases take extra work: a ratio within the 2e-5 band of the
// threshold (exactly rounded ratio) and an opened depth-cap bucket.
#pragma once

namespace nb {

// The interactions of a lane's two bodies with one source (its coordinates
// broadcast in both halves); m carries the source mass per body, zero where
// that body takes no interaction.
template <int LAW>
__device__ __forceinline__ void pair_accel_x2(float2 dx, float2 dy, float2 dz, float2 r2, float2 m, float2 S2,
                                              float2& ax, float2& ay, float2& az) {
    float2 w;
    if (LAW == NB_LAW_REFERENCE) {
        const float2 s = __fadd2_rn(r2, S2);
        const float2 t = __ffma2_rn(__fmul2_rn(r2, s), s, make_float2(kTravTiny, kTravTiny));
        w = __fmul2_rn(m, make_float2(rsqrt_approx(t.x), rsqrt_approx(t.y)));
    } else {
        const float2 q = __fadd2_rn(r2, S2);
        const float2 inv = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
        w = __fmul2_rn(__fmul2_rn(m, inv), __fmul2_rn(inv, inv));
    }
    ax = __ffma2_rn(w, dx, ax);
    ay = __ffma2_rn(w, dy, ay);
    az = __ffma2_rn(w, dz, az);
}

// Pairwise force of one body q of an opened depth-cap bucket on body p.
template <int LAW>
__device__ __forceinline__ void bucket_accel(const float4* __restrict__ spos, int first, int count, int n, int self,
                                             const float4 p, float S, float& ax, float& ay, float& az,
                                             unsigned& cnt) {
    const int qe = min(first + count, n);
    for (int q = max(first, 0); q < qe; ++q) {
        if (q == self) continue;
        const float4 bq = spos[q];
        const float dx = bq.x - p.x, dy = bq.y - p.y, dz = bq.z - p.z;
        pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), bq.w, S, ax, ay, az);
        ++cnt;
    }
}

template <int LAW>
__global__ void __launch_bounds__(kTravBlock) k_traverse(const float4* __restrict__ spos,
                                                         const int32_t* __restrict__ sorder, int n,
                                                         const float4* __restrict__ cell_com,
                                                         const int4* __restrict__ cell_meta,
                                                         const float4* __restrict__ cell_lo, int n_cells,
                                                         int max_pops, float theta_f, float S, float G,
                                                         float4* __restrict__ acc,
                                                         unsigned long long* __restrict__ inter,
                                                         int* __restrict__ err) {
    __shared__ int4 stk[kTravWarps][kStack];   // (child range, lanes for body slot 0, for slot 1, 0)
    __shared__ float4 kid_cm[kTravWarps][8];
    __shared__ int4 kid_mt[kTravWarps][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = (blockIdx.x * kTravWarps + w) * kTravBodies;
    const int s0 = base + lane, s1 = base + 32 + lane;
    const bool v0 = s0 < n, v1 = s1 < n;
    const float4 p0 = v0 ? spos[s0] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 p1 = v1 ? spos[s1] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 px = make_float2(p0.x, p1.x), py = make_float2(p0.y, p1.y), pz = make_float2(p0.z, p1.z);
    const float2 nx = make_float2(-p0.x, -p1.x), ny = make_float2(-p0.y, -p1.y), nz = make_float2(-p0.z, -p1.z);
    const float2 S2 = make_float2(S, S), z2 = make_float2(0.f, 0.f);
    float2 sx = z2, sy = z2, sz = z2, cx = z2, cy = z2, cz = z2, tx = z2, ty = z2, tz = z2;
    unsigned cnt = 0;
    int top = 0, pops = 0;
    bool bad = false;

    // Entry being processed: children [F, F + nch) opened by the lanes of m0 / m1.
    unsigned F = 0, nch = 1;
    unsigned m0 = __ballot_sync(0xffffffffu, v0), m1 = __ballot_sync(0xffffffffu, v1);
    while (true) {
        if ((int)lane < (int)nch) {
            kid_cm[w][lane] = __ldg(&cell_com[F + lane]);
            kid_mt[w][lane] = __ldg(&cell_meta[F + lane]);
        }
        __syncwarp();
        const bool a0 = (m0 >> lane) & 1u, a1 = (m1 >> lane) & 1u;
        for (unsigned j = 0; j < nch; ++j) {
            const float4 cm = kid_cm[w][j];
            const int4 mt = kid_mt[w][j];
            const int kind = mt.w & 15;
            if (kind == TK_SINGLE) {
                const bool i0 = a0 && mt.x != s0, i1 = a1 && mt.x != s1;
                if (i0 || i1) {
                    const float2 dx = __fadd2_rn(make_float2(cm.x, cm.x), nx);
                    const float2 dy = __fadd2_rn(make_float2(cm.y, cm.y), ny);
                    const float2 dz = __fadd2_rn(make_float2(cm.z, cm.z), nz);
                    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                    pair_accel_x2<LAW>(dx, dy, dz, r2, make_float2(i0 ? cm.w : 0.f, i1 ? cm.w : 0.f), S2, tx, ty, tz);
                    cnt += (i0 ? 1u : 0u) + (i1 ? 1u : 0u);
                }
                continue;
            }
            bool open0 = false, open1 = false;
            if (a0 || a1) {
                // the reference's float distance: dv = p - COM, r2 = (dvx^2 + dvy^2) + dvz^2, each op rounded
                const float2 dvx = __fadd2_rn(px, make_float2(-cm.x, -cm.x));
                const float2 dvy = __fadd2_rn(py, make_float2(-cm.y, -cm.y));
                const float2 dvz = __fadd2_rn(pz, make_float2(-cm.z, -cm.z));
                const float2 r2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(dvx, dvx), __fmul2_rn(dvy, dvy)), __fmul2_rn(dvz, dvz));
                const float thr_acc = __int_as_float(mt.y), thr_rej = __int_as_float(mt.z);
                bool acc0 = r2.x > thr_acc, acc1 = r2.y > thr_acc;
                if ((a0 && !acc0 && !(r2.x < thr_rej)) || (a1 && !acc1 && !(r2.y < thr_rej))) {
                    const float side = __ldg(&cell_lo[F + j]).w;
                    if (!acc0 && !(r2.x < thr_rej)) acc0 = __fdiv_rn(side, __fsqrt_rn(r2.x)) < theta_f;
                    if (!acc1 && !(r2.y < thr_rej)) acc1 = __fdiv_rn(side, __fsqrt_rn(r2.y)) < theta_f;
                }
                acc0 = acc0 && a0;
                acc1 = acc1 && a1;
                if ((acc0 || acc1) && cm.w != 0.f) {
                    pair_accel_x2<LAW>(make_float2(-dvx.x, -dvx.y), make_float2(-dvy.x, -dvy.y),
                                       make_float2(-dvz.x, -dvz.y), r2,
                                       make_float2(acc0 ? cm.w : 0.f, acc1 ? cm.w : 0.f), S2, tx, ty, tz);
                    cnt += (acc0 ? 1u : 0u) + (acc1 ? 1u : 0u);
                }
                if (kind == TK_INTERNAL) {
                    open0 = a0 && !acc0;
                    open1 = a1 && !acc1;
                } else {
                    // opened depth-cap bucket: each of its bodies except the body itself
                    const int bc = mt.w >> 8;
                    if (a0 && !acc0) bucket_accel<LAW>(spos, mt.x, bc, n, s0, p0, S, tx.x, ty.x, tz.x, cnt);
                    if (a1 && !acc1) bucket_accel<LAW>(spos, mt.x, bc, n, s1, p1, S, tx.y, ty.y, tz.y, cnt);
                }
            }
            const unsigned b0 = __ballot_sync(0xffffffffu, open0), b1 = __ballot_sync(0xffffffffu, open1);
            if (b0 | b1) {
                const unsigned cf = (unsigned)mt.x, cn = ((unsigned)mt.w >> 4) & 15u;
                if (top < kStack && cf < (1u << kRangeBits) && cn >= 1 && cn <= 8 && cf + cn <= (unsigned)n_cells) {
                    if (lane == 0) stk[w][top] = make_int4((int)(cf | (cn << kRangeBits)), (int)b0, (int)b1, 0);
                    ++top;
                } else {
                    bad = true;
                }
            }
        }
        kahan_add(sx.x, cx.x, tx.x); kahan_add(sy.x, cy.x, ty.x); kahan_add(sz.x, cz.x, tz.x);
        kahan_add(sx.y, cx.y, tx.y); kahan_add(sy.y, cy.y, ty.y); kahan_add(sz.y, cz.y, tz.y);
        tx = ty = tz = z2;
        // A well-formed tree pops each internal cell at most once per warp.
        if (bad || top == 0 || ++pops > max_pops) break;
        __syncwarp();
        --top;
        const int4 e = stk[w][top];
        F = (unsigned)e.x & ((1u << kRangeBits) - 1u);
        nch = (unsigned)e.x >> kRangeBits;
        m0 = (unsigned)e.y;
        m1 = (unsigned)e.z;
        __syncwarp();
    }
    if ((bad || top > 0) && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
    if (v0) acc[sorder[s0]] = make_float4(G * (sx.x - cx.x), G * (sy.x - cy.x), G * (sz.x - cz.x), 0.f);
    if (v1) acc[sorder[s1]] = make_float4(G * (sx.y - cx.y), G * (sy.y - cy.y), G * (sz.y - cz.y), 0.f);
    unsigned long long c = cnt;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(inter, c);
}

}  // namespace nb
