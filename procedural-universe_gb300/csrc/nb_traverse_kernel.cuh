// nb_traverse_kernel.cuh -- the K6 traversal kernel (included by nb_traverse.cu).
//
// A warp walks the tree for 64 consecutive bodies of the key order, two per
// lane (lane l holds bodies base + l and base + 32 + l).  Every body still
// makes exactly the decisions of the reference's recursion; what changes is
// where they are made:
//   * Each popped cell's children are first classified for the whole group
//     at once, one lane per child, from the group's bounding box: if even the
//     nearest point of the box is beyond the cell's accept distance, every
//     body of the group accepts the cell (its float r^2 exceeds the accept
//     threshold); if even the farthest corner is inside the reject distance,
//     every body opens it.  Both bounds carry a 1e-5 relative margin, far
//     above the few-ulp rounding of the float distances, so a group verdict
//     never differs from a body's own.
//   * Cells every body accepts, and one-body leaves, go to shared-memory lists
//     (with the lane masks of the bodies that reached them) that are evaluated
//     densely for both bodies of every lane with the packed FP32x2
//     instructions; cells every body opens are pushed without per-body work.
//   * Only the remaining ("ambiguous") cells and depth-cap buckets are decided
//     body by body, as the reference does, with the accept / reject
//     thresholds and the exactly rounded ratio inside the 2e-5 band.
// A stack entry carries one lane mask per body slot: the bodies that opened
// that cell.
#pragma once

namespace nb {

constexpr int kMultiTop = kStack - 176 - 32;   // stack height up to which a step takes several entries
static_assert(kMultiTop > 0, "stack too small for multi-entry steps");
constexpr int kListCells = 64;    // accepted cells waiting for evaluation, per warp
constexpr int kListBodies = 64;   // one-body leaves waiting for evaluation, per warp

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

// A source at c acting on the lane's two bodies (negated coordinates n*).
template <int LAW>
__device__ __forceinline__ void source_accel_x2(const float4 c, float2 m, float2 nx, float2 ny, float2 nz, float2 S2,
                                                float2& ax, float2& ay, float2& az) {
    const float2 dx = __fadd2_rn(make_float2(c.x, c.x), nx);
    const float2 dy = __fadd2_rn(make_float2(c.y, c.y), ny);
    const float2 dz = __fadd2_rn(make_float2(c.z, c.z), nz);
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    pair_accel_x2<LAW>(dx, dy, dz, r2, m, S2, ax, ay, az);
}

// Pairwise force of each body of an opened depth-cap bucket on body p.
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

enum : int { CL_NONE = -1, CL_SINGLE = 0, CL_ACCEPT = 1, CL_OPEN = 2, CL_DECIDE = 3, CL_EMPTY = 4 };

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
    // 12-byte entries (child range, lanes of body slot 0, of slot 1): the smaller the
    // shared-memory footprint, the more of the SM's L1 is left for the node reads
    struct StackEntry { int range, lanes0, lanes1; };
    __shared__ StackEntry stk[kTravWarps][kStack];
    __shared__ float4 kid_cm[kTravWarps][32];
    __shared__ int4 kid_mt[kTravWarps][32];
    __shared__ float4 lc_src[kTravWarps][kListCells];
    __shared__ uint2 lc_mask[kTravWarps][kListCells];
    __shared__ float4 lb_src[kTravWarps][kListBodies];
    __shared__ int4 lb_info[kTravWarps][kListBodies];   // (body index, mask slot 0, mask slot 1, 0)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const int base = (blockIdx.x * kTravWarps + w) * kTravBodies;
    const int s0 = base + lane, s1 = base + 32 + lane;
    const bool v0 = s0 < n, v1 = s1 < n;
    if (__ballot_sync(0xffffffffu, v0) == 0u) return;   // a warp past the last body (whole warp)
    const float4 p0 = v0 ? spos[s0] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 p1 = v1 ? spos[s1] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 nx = make_float2(-p0.x, -p1.x), ny = make_float2(-p0.y, -p1.y), nz = make_float2(-p0.z, -p1.z);
    const float2 S2 = make_float2(S, S), z2 = make_float2(0.f, 0.f);
    // the group's bounding box (valid bodies)
    float glo[3], ghi[3];
    {
        const float a0[3] = {p0.x, p0.y, p0.z}, a1[3] = {p1.x, p1.y, p1.z};
        for (int a = 0; a < 3; ++a) {
            glo[a] = fminf(v0 ? a0[a] : INFINITY, v1 ? a1[a] : INFINITY);
            ghi[a] = fmaxf(v0 ? a0[a] : -INFINITY, v1 ? a1[a] : -INFINITY);
            for (int o = 16; o > 0; o >>= 1) {
                glo[a] = fminf(glo[a], __shfl_xor_sync(0xffffffffu, glo[a], o));
                ghi[a] = fmaxf(ghi[a], __shfl_xor_sync(0xffffffffu, ghi[a], o));
            }
        }
    }
    float2 sx = z2, sy = z2, sz = z2, cx = z2, cy = z2, cz = z2, tx = z2, ty = z2, tz = z2;
    unsigned cnt = 0;
    // Lists fill from both ends: entries that every valid body of the warp
    // reached (and, for a body, not one of the warp's own) from the front,
    // evaluated without masks; the others from the back, with their masks.
    int top = 0, pops = 0, nclf = 0, nclp = 0, nbdf = 0, nbdp = 0;
    const unsigned vm0 = __ballot_sync(0xffffffffu, v0), vm1 = __ballot_sync(0xffffffffu, v1);
    bool bad = false;

    auto fold = [&]() {
        kahan_add(sx.x, cx.x, tx.x); kahan_add(sy.x, cy.x, ty.x); kahan_add(sz.x, cz.x, tz.x);
        kahan_add(sx.y, cx.y, tx.y); kahan_add(sy.y, cy.y, ty.y); kahan_add(sz.y, cz.y, tz.y);
        tx = ty = tz = z2;
    };
    auto flush_cells = [&]() {
        __syncwarp();
        for (int k = 0; k < nclf; ++k) {
            const float4 c = lc_src[w][k];
            source_accel_x2<LAW>(c, make_float2(c.w, c.w), nx, ny, nz, S2, tx, ty, tz);
        }
        for (int k = kListCells - nclp; k < kListCells; ++k) {
            const float4 c = lc_src[w][k];
            const uint2 mk = lc_mask[w][k];
            const float2 m = make_float2(((mk.x >> lane) & 1u) ? c.w : 0.f, ((mk.y >> lane) & 1u) ? c.w : 0.f);
            source_accel_x2<LAW>(c, m, nx, ny, nz, S2, tx, ty, tz);
        }
        nclf = nclp = 0;
        fold();
        __syncwarp();
    };
    auto flush_bodies = [&]() {
        __syncwarp();
        for (int k = 0; k < nbdf; ++k) {
            const float4 b = lb_src[w][k];
            source_accel_x2<LAW>(b, make_float2(b.w, b.w), nx, ny, nz, S2, tx, ty, tz);
        }
        for (int k = kListBodies - nbdp; k < kListBodies; ++k) {
            const float4 b = lb_src[w][k];
            const int4 bi = lb_info[w][k];
            const bool i0 = (((unsigned)bi.y >> lane) & 1u) && bi.x != s0;
            const bool i1 = (((unsigned)bi.z >> lane) & 1u) && bi.x != s1;
            source_accel_x2<LAW>(b, make_float2(i0 ? b.w : 0.f, i1 ? b.w : 0.f), nx, ny, nz, S2, tx, ty, tz);
        }
        nbdf = nbdp = 0;
        fold();
        __syncwarp();
    };

    // A walk step takes up to 8 entries from the top of the stack, as many as
    // have at most 32 children together; lane j handles the j-th of those
    // children (cell ch), reached by the bodies of its entry's masks (cm0, cm1).
    // The first step is the root, reached by every valid body.
    int T = 1;
    unsigned ch = 0;
    unsigned cm0 = __ballot_sync(0xffffffffu, v0), cm1 = __ballot_sync(0xffffffffu, v1);
    while (true) {
        // ---- classify the children for the whole group, one lane per child ----
        int cls = CL_NONE;
        float4 ccm = make_float4(0.f, 0.f, 0.f, 0.f);
        int4 cmt = make_int4(0, 0, 0, 0);
        if ((int)lane < T) {
            ccm = __ldg(&cell_com[ch]);
            cmt = __ldg(&cell_meta[ch]);
            kid_cm[w][lane] = ccm;
            kid_mt[w][lane] = cmt;
            const int kind = cmt.w & 15;
            if (kind == TK_SINGLE) {
                cls = CL_SINGLE;
            } else if (kind != TK_INTERNAL) {
                cls = CL_DECIDE;   // depth-cap bucket: body by body
            } else {
                const float c[3] = {ccm.x, ccm.y, ccm.z};
                float dmin2 = 0.f, dmax2 = 0.f;
                for (int a = 0; a < 3; ++a) {
                    // nearest and farthest point of the group's box along this axis
                    const float dn = fmaxf(0.f, fmaxf(glo[a] - c[a], c[a] - ghi[a]));
                    const float df = fmaxf(fabsf(ghi[a] - c[a]), fabsf(glo[a] - c[a]));
                    dmin2 = fmaf(dn, dn, dmin2);
                    dmax2 = fmaf(df, df, dmax2);
                }
                const float thr_acc = __int_as_float(cmt.y), thr_rej = __int_as_float(cmt.z);
                if (dmin2 * (1.f - 1e-5f) > thr_acc) cls = ccm.w != 0.f ? CL_ACCEPT : CL_EMPTY;
                else if (dmax2 * (1.f + 1e-5f) < thr_rej) cls = CL_OPEN;
                else cls = CL_DECIDE;
            }
        }
        __syncwarp();
        const unsigned bS = __ballot_sync(0xffffffffu, cls == CL_SINGLE);
        const unsigned bA = __ballot_sync(0xffffffffu, cls == CL_ACCEPT);
        const unsigned bO = __ballot_sync(0xffffffffu, cls == CL_OPEN);
        const unsigned bD = __ballot_sync(0xffffffffu, cls == CL_DECIDE);
        // one-body leaves: every body that reached them takes the pair (not the body itself)
        const bool reach_all = cm0 == vm0 && cm1 == vm1;
        if (bS) {
            if (nbdf + nbdp + __popc(bS) > kListBodies) flush_bodies();
            const int slot = cmt.x - base;
            const bool own = slot >= 0 && slot < kTravBodies;
            const unsigned bSf = __ballot_sync(0xffffffffu, cls == CL_SINGLE && reach_all && !own);
            if (cls == CL_SINGLE) {
                if ((bSf >> lane) & 1u) {
                    lb_src[w][nbdf + __popc(bSf & lt)] = ccm;
                } else {
                    const int k = kListBodies - 1 - (nbdp + __popc(bS & ~bSf & lt));
                    lb_src[w][k] = ccm;
                    lb_info[w][k] = make_int4(cmt.x, (int)cm0, (int)cm1, 0);
                }
                unsigned c2 = __popc(cm0) + __popc(cm1);
                if (own && (((slot < 32 ? cm0 : cm1) >> (slot & 31)) & 1u)) --c2;
                cnt += c2;
            }
            nbdf += __popc(bSf);
            nbdp += __popc(bS & ~bSf);
        }
        // cells every body accepts: the monopole, for every body that reached them
        if (bA) {
            if (nclf + nclp + __popc(bA) > kListCells) flush_cells();
            const unsigned bAf = __ballot_sync(0xffffffffu, cls == CL_ACCEPT && reach_all);
            if (cls == CL_ACCEPT) {
                if ((bAf >> lane) & 1u) {
                    lc_src[w][nclf + __popc(bAf & lt)] = ccm;
                } else {
                    const int k = kListCells - 1 - (nclp + __popc(bA & ~bAf & lt));
                    lc_src[w][k] = ccm;
                    lc_mask[w][k] = make_uint2(cm0, cm1);
                }
                cnt += __popc(cm0) + __popc(cm1);
            }
            nclf += __popc(bAf);
            nclp += __popc(bA & ~bAf);
        }
        // cells every body opens
        if (bO) {
            bool ok = true;
            if (cls == CL_OPEN) {
                const unsigned cf = (unsigned)cmt.x, cn = ((unsigned)cmt.w >> 4) & 15u;
                ok = cf < (1u << kRangeBits) && cn >= 1 && cn <= 8 && cf + cn <= (unsigned)n_cells;
                if (ok && top + __popc(bO) <= kStack)
                    stk[w][top + __popc(bO & lt)] = StackEntry{(int)(cf | (cn << kRangeBits)), (int)cm0, (int)cm1};
            }
            if (!__all_sync(0xffffffffu, ok) || top + __popc(bO) > kStack) bad = true;
            top += __popc(bO);
        }
        // the rest: each body decides, as the reference's recursion does
        __syncwarp();
        // Two ambiguous children per iteration: their arithmetic is independent,
        // so the two dependency chains interleave; the stack receives the first
        // child's entry before the second's, as one child per iteration would.
        auto decide = [&](int j, unsigned pm0, unsigned pm1, unsigned chj, bool& open0, bool& open1) {
            const float4 cm = kid_cm[w][j];
            const int4 mt = kid_mt[w][j];
            const bool a0 = (pm0 >> lane) & 1u, a1 = (pm1 >> lane) & 1u;
            // the reference's float distance: dv = p - COM, r2 = (dvx^2 + dvy^2) + dvz^2, each op
            // rounded; d = COM - p = -dv exactly (rounding is symmetric), so r2 is the same
            const float2 dx = __fadd2_rn(make_float2(cm.x, cm.x), nx);
            const float2 dy = __fadd2_rn(make_float2(cm.y, cm.y), ny);
            const float2 dz = __fadd2_rn(make_float2(cm.z, cm.z), nz);
            const float2 r2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
            const float thr_acc = __int_as_float(mt.y), thr_rej = __int_as_float(mt.z);
            bool acc0 = r2.x > thr_acc, acc1 = r2.y > thr_acc;
            const bool band0 = a0 && !acc0 && !(r2.x < thr_rej), band1 = a1 && !acc1 && !(r2.y < thr_rej);
            if (band0 || band1) {
                const float side = __ldg(&cell_lo[chj]).w;
                if (band0) acc0 = __fdiv_rn(side, __fsqrt_rn(r2.x)) < theta_f;
                if (band1) acc1 = __fdiv_rn(side, __fsqrt_rn(r2.y)) < theta_f;
            }
            acc0 = acc0 && a0;
            acc1 = acc1 && a1;
            // a body that does not take the cell adds an exact zero (zero mass, finite factor)
            pair_accel_x2<LAW>(dx, dy, dz, r2, make_float2(acc0 ? cm.w : 0.f, acc1 ? cm.w : 0.f), S2, tx, ty, tz);
            if (cm.w != 0.f) cnt += (acc0 ? 1u : 0u) + (acc1 ? 1u : 0u);
            const int kind = mt.w & 15;
            if (kind == TK_INTERNAL) {
                open0 = a0 && !acc0;
                open1 = a1 && !acc1;
            } else {
                // opened depth-cap bucket: each of its bodies except the body itself
                const int bc = mt.w >> 8;
                if (a0 && !acc0) bucket_accel<LAW>(spos, mt.x, bc, n, s0, p0, S, tx.x, ty.x, tz.x, cnt);
                if (a1 && !acc1) bucket_accel<LAW>(spos, mt.x, bc, n, s1, p1, S, tx.y, ty.y, tz.y, cnt);
                open0 = open1 = false;
            }
        };
        auto push = [&](int j, bool open0, bool open1) {
            const unsigned b0 = __ballot_sync(0xffffffffu, open0), b1 = __ballot_sync(0xffffffffu, open1);
            if (b0 | b1) {
                const int4 mt = kid_mt[w][j];
                const unsigned cf = (unsigned)mt.x, cn = ((unsigned)mt.w >> 4) & 15u;
                if (top < kStack && cf < (1u << kRangeBits) && cn >= 1 && cn <= 8 && cf + cn <= (unsigned)n_cells) {
                    if (lane == 0) stk[w][top] = StackEntry{(int)(cf | (cn << kRangeBits)), (int)b0, (int)b1};
                    ++top;
                } else {
                    bad = true;
                }
            }
        };
        for (unsigned rem = bD; rem && !bad;) {
            const int j = __ffs(rem) - 1;
            rem &= rem - 1u;
            const bool two = rem != 0u;   // warp-uniform
            const int k = two ? __ffs(rem) - 1 : j;
            if (two) rem &= rem - 1u;
            const unsigned pj0 = __shfl_sync(0xffffffffu, cm0, j), pj1 = __shfl_sync(0xffffffffu, cm1, j);
            const unsigned chj = __shfl_sync(0xffffffffu, ch, j);
            const unsigned pk0 = __shfl_sync(0xffffffffu, cm0, k), pk1 = __shfl_sync(0xffffffffu, cm1, k);
            const unsigned chk = __shfl_sync(0xffffffffu, ch, k);
            bool oj0, oj1, ok0, ok1;
            decide(j, pj0, pj1, chj, oj0, oj1);
            decide(k, two ? pk0 : 0u, two ? pk1 : 0u, chk, ok0, ok1);
            push(j, oj0, oj1);
            if (two && !bad) push(k, ok0, ok1);
        }
        fold();
        // A well-formed tree pushes each internal cell at most once per warp.
        if (bad || top == 0 || ++pops > max_pops) break;
        // ---- next step: up to 8 entries from the top of the stack ----
        // A step pushes at most 32 entries.  Above kMultiTop entries the walk
        // takes one entry per step, a depth-first walk that leaves at most 7
        // entries per tree level (7 * 21 + 8 in all), so the stack never holds
        // more than kMultiTop + 31 + 155 < kStack entries.
        __syncwarp();
        const int cap = top <= kMultiTop ? 8 : 1;
        unsigned eF = 0, em0 = 0, em1 = 0;
        int en = 0;
        if (lane < cap && lane < top) {
            const StackEntry e = stk[w][top - 1 - lane];
            eF = (unsigned)e.range & ((1u << kRangeBits) - 1u);
            en = (int)((unsigned)e.range >> kRangeBits);
            em0 = (unsigned)e.lanes0;
            em1 = (unsigned)e.lanes1;
        }
        int incl = en;   // inclusive prefix of the child counts over lanes 0..7
        for (int o = 1; o < 8; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const unsigned take = __ballot_sync(0xffffffffu, lane < cap && lane < top && incl <= 32);
        const int P = __popc(take);   // >= 1: an entry has at most 8 children
        T = __shfl_sync(0xffffffffu, incl, P - 1);
        __syncwarp();
        top -= P;
        // this lane's entry: the last taken entry whose children start at or
        // before it (every entry has at least one child, so the starts differ)
        const unsigned starts = __reduce_or_sync(0xffffffffu, lane < P ? 1u << (incl - en) : 0u);
        const int q = (__popc(starts & ((2u << lane) - 1u)) - 1) & 7;
        const unsigned qF = __shfl_sync(0xffffffffu, eF, q);
        const int qx = __shfl_sync(0xffffffffu, incl - en, q);
        cm0 = __shfl_sync(0xffffffffu, em0, q);
        cm1 = __shfl_sync(0xffffffffu, em1, q);
        ch = qF + (unsigned)(lane - qx);
    }
    if (!bad) {
        flush_cells();
        flush_bodies();
    }
    if ((bad || top > 0) && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
    if (v0) acc[sorder[s0]] = make_float4(G * (sx.x - cx.x), G * (sy.x - cy.x), G * (sz.x - cz.x), 0.f);
    if (v1) acc[sorder[s1]] = make_float4(G * (sx.y - cx.y), G * (sy.y - cy.y), G * (sz.y - cz.y), 0.f);
    unsigned long long c = cnt;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(inter, c);
}

}  // namespace nb
