// nb_traverse_kernel.cuh -- the K6 traversal kernel (included by nb_traverse.cu).
//
// One body per lane.  Lanes outside the popped entry's mask skip the child
// work through a divergent branch; when no lane of the warp accepts a child
// (near the bodies, every lane opens) the warp skips the force altogether.
// Only the rare cases take extra work: a ratio within the 2e-5 band of the
// threshold (exactly rounded ratio) and an opened depth-cap bucket.
#pragma once

namespace nb {

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
    __shared__ int2 stk[kTravWarps][kStack];
    __shared__ float4 kid_cm[kTravWarps][8];
    __shared__ int4 kid_mt[kTravWarps][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = (blockIdx.x * kTravWarps + w) * 32 + lane;
    const bool valid = s < n;
    const float4 p = valid ? spos[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    unsigned cnt = 0;
    int top = 0, pops = 0;
    bool bad = false;

    // Entry being processed: children [F, F + nch) opened by the lanes of `mask`.
    unsigned F = 0, nch = 1, mask = __ballot_sync(0xffffffffu, valid);   // the root, child of a virtual node
    while (true) {
        if ((int)lane < (int)nch) {
            kid_cm[w][lane] = __ldg(&cell_com[F + lane]);
            kid_mt[w][lane] = __ldg(&cell_meta[F + lane]);
        }
        __syncwarp();
        const bool mine = (mask >> lane) & 1u;
        for (unsigned j = 0; j < nch; ++j) {
            const float4 cm = kid_cm[w][j];
            const int4 mt = kid_mt[w][j];
            const int kind = mt.w & 15;
            if (kind == TK_SINGLE) {
                if (mine && mt.x != s) {
                    const float dx = cm.x - p.x, dy = cm.y - p.y, dz = cm.z - p.z;
                    pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), cm.w, S, tx, ty, tz);
                    ++cnt;
                }
                continue;
            }
            bool open = false;
            if (mine) {
                const float dvx = __fsub_rn(p.x, cm.x), dvy = __fsub_rn(p.y, cm.y), dvz = __fsub_rn(p.z, cm.z);
                const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dvx, dvx), __fmul_rn(dvy, dvy)), __fmul_rn(dvz, dvz));
                bool accept = r2 > __int_as_float(mt.y);
                if (!accept && !(r2 < __int_as_float(mt.z))) {
                    const float side = __ldg(&cell_lo[F + j]).w;
                    accept = __fdiv_rn(side, __fsqrt_rn(r2)) < theta_f;
                }
                if (accept) {
                    if (cm.w != 0.f) {
                        pair_accel<LAW>(-dvx, -dvy, -dvz, r2, cm.w, S, tx, ty, tz);
                        ++cnt;
                    }
                } else if (kind == TK_INTERNAL) {
                    open = true;
                } else {
                    // opened depth-cap bucket: each of its bodies except the lane's own
                    const int qe = min(mt.x + (mt.w >> 8), n);
                    for (int q = max(mt.x, 0); q < qe; ++q) {
                        if (q == s) continue;
                        const float4 bq = spos[q];
                        const float dx = bq.x - p.x, dy = bq.y - p.y, dz = bq.z - p.z;
                        pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), bq.w, S, tx, ty, tz);
                        ++cnt;
                    }
                }
            }
            const unsigned b = __ballot_sync(0xffffffffu, open);
            if (b) {
                const unsigned cf = (unsigned)mt.x, cn = ((unsigned)mt.w >> 4) & 15u;
                if (top < kStack && cf < (1u << kRangeBits) && cn >= 1 && cn <= 8 && cf + cn <= (unsigned)n_cells) {
                    if (lane == 0) stk[w][top] = make_int2((int)(cf | (cn << kRangeBits)), (int)b);
                    ++top;
                } else {
                    bad = true;
                }
            }
        }
        kahan_add(sx, cx, tx);
        kahan_add(sy, cy, ty);
        kahan_add(sz, cz, tz);
        tx = ty = tz = 0.f;
        // A well-formed tree pops each internal cell at most once per warp.
        if (bad || top == 0 || ++pops > max_pops) break;
        __syncwarp();
        --top;
        const int2 e = stk[w][top];
        F = (unsigned)e.x & ((1u << kRangeBits) - 1u);
        nch = (unsigned)e.x >> kRangeBits;
        mask = (unsigned)e.y;
        __syncwarp();
    }
    if ((bad || top > 0) && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
    if (valid) acc[sorder[s]] = make_float4(G * (sx - cx), G * (sy - cy), G * (sz - cz), 0.f);
    unsigned long long c = cnt;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(inter, c);
}

}  // namespace nb
