// nb_traverse_kernel.cuh -- the K6 traversal kernel (included by nb_traverse.cu).
//
// BPL bodies per lane: a warp owns 32 * BPL consecutive bodies of the sorted
// order, lane l holding bodies base + l + 32 b (b < BPL).  Each stack entry
// carries one lane mask per body slot, so every body keeps its own opening
// decisions; the per-visit work of loading a child and branching on its kind
// is shared by BPL bodies.
#pragma once

namespace nb {

template <int LAW, int BPL>
__global__ void __launch_bounds__(kTravBlock) k_traverse(const float4* __restrict__ spos,
                                                         const int32_t* __restrict__ sorder, int n,
                                                         const float4* __restrict__ cell_com,
                                                         const int4* __restrict__ cell_meta,
                                                         const float4* __restrict__ cell_lo, int n_cells,
                                                         int max_pops, float theta_f, float S, float G,
                                                         float4* __restrict__ acc,
                                                         unsigned long long* __restrict__ inter,
                                                         int* __restrict__ err) {
    __shared__ int4 stk[kTravWarps][kStack];
    __shared__ float4 kid_cm[kTravWarps][8];
    __shared__ int4 kid_mt[kTravWarps][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = (blockIdx.x * kTravWarps + w) * 32 * BPL + lane;
    int sidx[BPL];
    float4 p[BPL];
    float sx[BPL], sy[BPL], sz[BPL], cx[BPL], cy[BPL], cz[BPL], tx[BPL], ty[BPL], tz[BPL];
    unsigned mask[BPL];
    unsigned cnt = 0;
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        sidx[b] = base + 32 * b;
        const bool v = sidx[b] < n;
        p[b] = v ? spos[sidx[b]] : make_float4(0.f, 0.f, 0.f, 0.f);
        sx[b] = sy[b] = sz[b] = cx[b] = cy[b] = cz[b] = tx[b] = ty[b] = tz[b] = 0.f;
        mask[b] = __ballot_sync(0xffffffffu, v);   // the root, as the child of a virtual node
    }
    int top = 0, pops = 0;
    bool bad = false;
    unsigned F = 0, nch = 1;
    while (true) {
        if ((int)lane < (int)nch) {
            kid_cm[w][lane] = __ldg(&cell_com[F + lane]);
            kid_mt[w][lane] = __ldg(&cell_meta[F + lane]);
        }
        __syncwarp();
        bool mine[BPL];
#pragma unroll
        for (int b = 0; b < BPL; ++b) mine[b] = (mask[b] >> lane) & 1u;
        for (unsigned j = 0; j < nch; ++j) {
            const float4 cm = kid_cm[w][j];
            const int4 mt = kid_mt[w][j];
            const int kind = mt.w & 15;
            if (kind == TK_SINGLE) {
#pragma unroll
                for (int b = 0; b < BPL; ++b) {
                    if (mine[b] && mt.x != sidx[b]) {
                        const float dx = cm.x - p[b].x, dy = cm.y - p[b].y, dz = cm.z - p[b].z;
                        pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), cm.w, S, tx[b], ty[b],
                                        tz[b]);
                        ++cnt;
                    }
                }
                continue;
            }
            unsigned ob[BPL];
            unsigned any = 0;
#pragma unroll
            for (int b = 0; b < BPL; ++b) {
                bool open = false;
                if (mine[b]) {
                    const float dvx = __fsub_rn(p[b].x, cm.x), dvy = __fsub_rn(p[b].y, cm.y),
                                dvz = __fsub_rn(p[b].z, cm.z);
                    const float r2 =
                        __fadd_rn(__fadd_rn(__fmul_rn(dvx, dvx), __fmul_rn(dvy, dvy)), __fmul_rn(dvz, dvz));
                    bool accept = r2 > __int_as_float(mt.y);
                    if (!accept && !(r2 < __int_as_float(mt.z))) {
                        const float side = __ldg(&cell_lo[F + j]).w;
                        accept = __fdiv_rn(side, __fsqrt_rn(r2)) < theta_f;
                    }
                    if (accept) {
                        if (cm.w != 0.f) {
                            pair_accel<LAW>(-dvx, -dvy, -dvz, r2, cm.w, S, tx[b], ty[b], tz[b]);
                            ++cnt;
                        }
                    } else if (kind == TK_INTERNAL) {
                        open = true;
                    } else {
                        const int qe = min(mt.x + (mt.w >> 8), n);
                        for (int q = max(mt.x, 0); q < qe; ++q) {
                            if (q == sidx[b]) continue;
                            const float4 bq = spos[q];
                            const float dx = bq.x - p[b].x, dy = bq.y - p[b].y, dz = bq.z - p[b].z;
                            pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), bq.w, S, tx[b], ty[b],
                                            tz[b]);
                            ++cnt;
                        }
                    }
                }
                ob[b] = __ballot_sync(0xffffffffu, open);
                any |= ob[b];
            }
            if (any) {
                const unsigned cf = (unsigned)mt.x, cn = ((unsigned)mt.w >> 4) & 15u;
                if (top < kStack && cf < (1u << kRangeBits) && cn >= 1 && cn <= 8 && cf + cn <= (unsigned)n_cells) {
                    if (lane == 0)
                        stk[w][top] = make_int4((int)(cf | (cn << kRangeBits)), (int)ob[0], BPL > 1 ? (int)ob[BPL - 1] : 0, 0);
                    ++top;
                } else {
                    bad = true;
                }
            }
        }
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            kahan_add(sx[b], cx[b], tx[b]);
            kahan_add(sy[b], cy[b], ty[b]);
            kahan_add(sz[b], cz[b], tz[b]);
            tx[b] = ty[b] = tz[b] = 0.f;
        }
        // A well-formed tree pops each internal cell at most once per warp.
        if (bad || top == 0 || ++pops > max_pops) break;
        __syncwarp();
        --top;
        const int4 e = stk[w][top];
        F = (unsigned)e.x & ((1u << kRangeBits) - 1u);
        nch = (unsigned)e.x >> kRangeBits;
        mask[0] = (unsigned)e.y;
        if (BPL > 1) mask[BPL - 1] = (unsigned)e.z;
        __syncwarp();
    }
    if ((bad || top > 0) && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
#pragma unroll
    for (int b = 0; b < BPL; ++b)
        if (sidx[b] < n)
            acc[sorder[sidx[b]]] = make_float4(G * (sx[b] - cx[b]), G * (sy[b] - cy[b]), G * (sz[b] - cz[b]), 0.f);
    unsigned long long c = cnt;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(inter, c);
}

}  // namespace nb
