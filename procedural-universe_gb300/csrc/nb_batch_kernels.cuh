// nb_batch_kernels.cuh -- kernels of the batched form (included by nb_batch.cu).
//
// Many independent galaxies are stepped together, one launch per phase:
//  * Barnes-Hut members (n >= threshold) are stored first, contiguously.  Each
//    gets a tight bounding cube; a body's key is its galaxy slot (21 bits, the
//    top 7 octal levels) followed by a 42-bit Morton code in its cube (14
//    levels), so ONE radix sort and ONE topology build make a forest whose
//    level-7 nodes are the galaxy roots.
//  * The mass pass adds traceless quadrupole moments (parallel-axis rule
//    bottom-up); a cell's centre of mass, walk record and quadrupole form one
//    64-byte record (nb_cellrec.cuh).  Traversal groups are
//    taken from the tree itself: the largest subtrees of at most kGroupMax
//    bodies whose cell is at most 1/16 of the galaxy cube, consecutive small
//    siblings packed together, oversized depth-cap buckets cut into chunks --
//    so a group is spatially compact and its bounding box small.  A warp
//    takes groups from a device queue (two bodies per lane; one for groups of
//    at most 32 bodies, so that half-empty warps do no idle work), opens a
//    cell when the cell side exceeds theta times the distance from the cell's
//    centre of mass to the group's bounding box, and collects accepted cells
//    (monopole + quadrupole) and leaf buckets of at most leaf_size bodies
//    (summed body by body) in shared-memory lists that every lane then
//    evaluates for its bodies with the packed FP32x2 instructions; accepted
//    cells far from the group go into the group's local expansion instead.
//    This is a performance form whose parity is the force error against the
//    FP64 direct sum (<= 1e-3), not the reference's per-body opening rule.
//  * Direct-sum members are padded to multiples of 256 bodies; a persistent
//    kernel takes (galaxy, target block, source range) units from a table
//    through an atomic counter, and a second kernel folds the partials.
#pragma once

#include <type_traits>

#include "nb_morton.cuh"
#include "nb_cellrec.cuh"

namespace nb {

constexpr int kGWarps = 4;              // warps per traversal block
constexpr int kGroupMax = 64;           // bodies per traversal group (two per lane)
constexpr int kGroupMinDepth = 4;       // a group cell lies >= 4 levels below its galaxy root
constexpr int kBoxChunk = 8192;         // bodies per block of the bounding-box pass
constexpr int kGStack = 512;            // cells waiting to be opened, per warp (<= 32 pushed per step)
constexpr int kStackCellLimit = 1 << 27;   // a stack entry packs a first-child index below this with 4 bits
constexpr int kGMultiTop = kGStack - 155 - 32;   // stack height up to which a walk step takes several cells
constexpr int kGCells = 64;             // accepted-cell list, per warp
constexpr int kGBodies = 192;           // gathered leaf-bucket bodies, per warp
constexpr int kDirTile = 128;           // sources per shared tile of the batched direct kernel
// far-field defaults of the group traversal (rules in nb_batch.cu's nb_batch)
constexpr double kFarEta = 0.2;         // geometric rule: group half-diagonal / distance
constexpr double kFarAlpha = 1e-4;      // relative rule: truncation estimate / (|a|_min / G)
constexpr double kFarCap = 0.5;         // relative rule: largest half-diagonal / distance


// ---- per-body galaxy tables -------------------------------------------------
constexpr int kFillChunk = 8192;   // bodies per block of the table fill
// run = (first entry, entries, value, table): table 0 is the Barnes-Hut bodies'
// slot, table 1 the direct-sum bodies' galaxy.
__global__ void k_fill_tables(const int4* __restrict__ runs, int32_t* __restrict__ slot, int32_t* __restrict__ dgal) {
    const int4 r = runs[blockIdx.x];
    int32_t* out = r.w ? dgal : slot;
    for (int i = threadIdx.x; i < r.y; i += blockDim.x) out[r.x + i] = r.z;
}

// ---- bounding cube of each Barnes-Hut galaxy ------------------------------
// Min/max are exact and order-free, so chunks of kBoxChunk bodies reduce in
// parallel into per-galaxy words with atomics on an order-preserving integer
// image of the float (nb_morton.cuh).
//
// The first kernel of a batched step also clears the step's counters: the
// tree counters and the radix histograms (TC_NIN set to the bodies in the
// forest), the interaction count, the traversal group counters and the
// direct-sum unit counter.
__global__ void k_gal_box_init(unsigned* __restrict__ bits, int nslot, int32_t* __restrict__ counters,
                               int counter_words, int n_in, unsigned long long* __restrict__ interactions,
                               int* __restrict__ group_ctr, int* __restrict__ next_unit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * nslot) bits[i] = (i % 6) < 3 ? 0xffffffffu : 0u;
    for (int j = i; j < counter_words; j += gridDim.x * blockDim.x) counters[j] = j == TC_NIN ? n_in : 0;
    if (i == 0) {
        *interactions = 0ull;
        group_ctr[0] = group_ctr[1] = 0;
        if (next_unit) *next_unit = 0;
    }
}

__device__ __forceinline__ void box_flush(unsigned* bits, int slot, const float lo[3], const float hi[3]) {
    for (int a = 0; a < 3; ++a) {
        atomicMin(&bits[6 * slot + a], float_to_ordered(lo[a]));
        atomicMax(&bits[6 * slot + 3 + a], float_to_ordered(hi[a]));
    }
}

// block b reduces bodies [b*kBoxChunk, (b+1)*kBoxChunk) of the Barnes-Hut range
__global__ void __launch_bounds__(256) k_gal_box_chunks(const float4* __restrict__ pos,
                                                        const int32_t* __restrict__ body_slot, int n, int nslot,
                                                        unsigned* __restrict__ bits) {
    const int base = blockIdx.x * kBoxChunk;
    const int end = min(n, base + kBoxChunk);
    int cur = -1;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = base + threadIdx.x; i < end; i += blockDim.x) {
        const int s = body_slot[i];
        if (s < 0 || s >= nslot) continue;
        if (s != cur) {
            if (cur >= 0) box_flush(bits, cur, lo, hi);
            cur = s;
            lo[0] = lo[1] = lo[2] = INFINITY;
            hi[0] = hi[1] = hi[2] = -INFINITY;
        }
        const float4 p = pos[i];
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
    // common case: the whole warp ended in one galaxy -> one set of atomics per warp
    const int lane = threadIdx.x & 31;
    const int c0 = __shfl_sync(0xffffffffu, cur, 0);
    if (__all_sync(0xffffffffu, cur == c0)) {
        for (int a = 0; a < 3; ++a)
            for (int o = 16; o > 0; o >>= 1) {
                lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
                hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
            }
        if (lane == 0 && c0 >= 0) box_flush(bits, c0, lo, hi);
    } else if (cur >= 0) {
        box_flush(bits, cur, lo, hi);
    }
}

// ---- bottom-up mass, centre of mass and quadrupole --------------------------
// Q_ij = sum m (3 y_i y_j - |y|^2 d_ij), y = offset from the node's centre of
// mass; a parent sums its children's Q plus m_c (3 d d - |d|^2 I), d = com_c - com.
// Leaf records are written by the placement (nb_cellrec.cuh); an internal
// node reads its children's records (contiguous) and writes its own whole.
__device__ void finish_moments(int k, const int32_t* int_cell, const int32_t* int_block, const uint32_t* int_mask,
                               const int32_t* int_first, const int32_t* int_level, CellRec* rec, int cell_cap,
                               int* err) {
    const int c = int_cell[k];
    const int F = 1 + int_block[k];
    const int nch = __popc(int_mask[k]);
    if (c < 0 || c >= cell_cap || F + nch > cell_cap) {   // corrupt node: report, never dereference
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    float4 ccm[8], cq1[8], cq2[8];
    float m = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    int count = 0;
    for (int j = 0; j < nch; ++j) {
        const CellRec* r = rec + F + j;
        ccm[j] = __ldcg(&r->com);
        count += __ldcg(&r->walk).y;
        cq1[j] = __ldcg(&r->q1);
        cq2[j] = __ldcg(&r->q2);
        m += ccm[j].w;
        cx = fmaf(ccm[j].w, ccm[j].x, cx); cy = fmaf(ccm[j].w, ccm[j].y, cy); cz = fmaf(ccm[j].w, ccm[j].z, cz);
    }
    const float im = m > 0.f ? 1.f / m : 0.f;
    cx *= im; cy *= im; cz *= im;
    float xx = 0.f, yy = 0.f, zz = 0.f, xy = 0.f, xz = 0.f, yz = 0.f;
    for (int j = 0; j < nch; ++j) {
        const float mc = ccm[j].w;
        const float dx = ccm[j].x - cx, dy = ccm[j].y - cy, dz = ccm[j].z - cz, r2 = dx * dx + dy * dy + dz * dz;
        xx += cq1[j].x + mc * (3.f * dx * dx - r2);
        yy += cq1[j].y + mc * (3.f * dy * dy - r2);
        zz += cq1[j].z + mc * (3.f * dz * dz - r2);
        xy += cq2[j].x + mc * 3.f * dx * dy;
        xz += cq2[j].y + mc * 3.f * dx * dz;
        yz += cq2[j].z + mc * 3.f * dy * dz;
    }
    CellRec* r = rec + c;
    __stcg(&r->com, make_float4(cx, cy, cz, m));
    __stcg(&r->walk, walk_record(F, count, int_first[k], BK_INTERNAL, nch, int_level[k]));
    __stcg(&r->q1, make_float4(xx, yy, zz, 0.f));
    __stcg(&r->q2, make_float4(xy, xz, yz, 0.f));
}

// One thread per internal node whose children are all leaves; the last child
// of a node to finish finishes the node (acquire-release counter per node).
__global__ void k_batch_moments(int int_cap, const int32_t* __restrict__ counters,
                                const int32_t* __restrict__ int_parent, const int32_t* __restrict__ int_nint,
                                int32_t* __restrict__ int_pending, const int32_t* __restrict__ int_cell,
                                const int32_t* __restrict__ int_block, const uint32_t* __restrict__ int_mask,
                                const int32_t* __restrict__ int_first, const int32_t* __restrict__ int_level,
                                CellRec* __restrict__ rec, int cell_cap, int* __restrict__ err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (!tree_fits(counters, int_cap, cell_cap)) return;   // held step: no moments
    const int ni = min(counters[TC_NINT], int_cap);
    if (k >= ni || int_nint[k] != 0) return;
    for (int guard = 0; guard < 64; ++guard) {
        finish_moments(k, int_cell, int_block, int_mask, int_first, int_level, rec, cell_cap, err);
        if (k == 0) return;
        const int p = int_parent[k];
        if (p < 0 || p >= ni) return;
        const int old = atomic_add_acq_rel(&int_pending[p], 1);   // publishes this node, sees its siblings
        if (old != int_nint[p] - 1) return;
        k = p;
    }
}

// Root cell of each galaxy: the level-7 internal node starting at the
// galaxy's first sorted position.
__global__ void k_batch_roots(const int32_t* __restrict__ slot_start, int nslot, const uint64_t* __restrict__ keys,
                              const int32_t* __restrict__ int_base, const int32_t* __restrict__ int_cell,
                              const int32_t* __restrict__ counters, int int_cap, int cell_cap,
                              int32_t* __restrict__ root, int32_t* __restrict__ err) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nslot) return;
    if (!tree_fits(counters, int_cap, cell_cap)) return;   // held step: no walk
    const int s = slot_start[g];
    int prev = -1;
    if (s > 0) {
        const uint64_t x = keys[s - 1] ^ keys[s];
        prev = x == 0 ? kBatchDepth : (__clzll((long long)x) - (64 - 3 * kBatchDepth)) / 3;
    }
    const int k = int_base[s] + (kSlotLevels - (prev + 1));
    if (prev + 1 > kSlotLevels || k < 0 || k >= min(counters[TC_NINT], int_cap)) {
        root[g] = -1;
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    root[g] = int_cell[k];
}

// ---- traversal groups from the tree --------------------------------------------
// One thread per internal node at or below the galaxy roots.  A node that
// cannot be a group itself emits its children that can (packing consecutive
// ones, children being contiguous in sorted order, when the node is deep
// enough), emits a body that sits high in the tree on its own and cuts a
// larger depth-cap bucket into chunks; internal children that cannot be
// groups are handled by their own threads.  Every body lands in exactly one
// group: the first groupable cell on its path from the galaxy root, or its
// leaf.
__device__ __forceinline__ void emit_group(int first, int count, const int32_t* sorder, const int32_t* body_slot,
                                           int nbodies, int4* groups, int cap, int* n_groups, int* err) {
    if (count <= 0) return;
    if (first < 0 || first + count > nbodies) {
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    const int idx = atomicAdd(n_groups, 1);
    if (idx >= cap) {
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    groups[idx] = make_int4(body_slot[sorder[first]], first, count, 0);
}

// A cell can be a group when it holds at most kGroupMax bodies and lies at
// least kGroupMinDepth levels below its galaxy's root (side <= cube / 16): a
// few bodies spread over a large, sparse cell would give one group a box the
// size of the galaxy and a list of ~10^5 entries (a tail that held one warp
// for milliseconds); such cells are split further instead.
__device__ __forceinline__ bool groupable(int level, int count) {
    return count <= kGroupMax && level >= kSlotLevels + kGroupMinDepth;
}

__global__ void k_batch_groups(int int_cap, const int32_t* __restrict__ counters, const int32_t* __restrict__ int_cell,
                               const CellRec* __restrict__ rec, const int32_t* __restrict__ sorder,
                               const int32_t* __restrict__ body_slot, int n_cells, int nbodies,
                               int4* __restrict__ groups, int cap, int* __restrict__ n_groups, int* __restrict__ err) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    // a held step emits no groups, so the traversal after it has no work
    if (!tree_fits(counters, int_cap, n_cells)) return;
    if (k >= min(counters[TC_NINT], int_cap)) return;
    const int c = int_cell[k];
    if (c < 0 || c >= n_cells) {
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    const int4 wr = rec[c].walk;
    const int level = wr.w >> 8;
    const int cnt = wr.y;
    if (level < kSlotLevels) return;
    if (groupable(level, cnt)) return;   // its parent groups it
    const int F = wr.x, nch = (wr.w >> 4) & 15;
    if (F < 1 || nch > 8 || F + nch > n_cells) {
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    // siblings are packed only below a cell small enough to be a group itself
    const bool pack = level >= kSlotLevels + kGroupMinDepth;
    int run_first = -1, run_cnt = 0;
    for (int j = 0; j < nch; ++j) {
        const int ch = F + j;
        const int4 cw = rec[ch].walk;
        const int kind = cw.w & 15;
        const int cc = cw.y;
        const int cf = cw.z;
        if (!groupable(cw.w >> 8, cc)) {
            emit_group(run_first, run_cnt, sorder, body_slot, nbodies, groups, cap, n_groups, err);
            run_first = -1;
            run_cnt = 0;
            if (kind != BK_INTERNAL)   // a body high in the tree, or an oversized depth-cap bucket
                for (int o = 0; o < cc; o += kGroupMax)
                    emit_group(cf + o, min(kGroupMax, cc - o), sorder, body_slot, nbodies, groups, cap, n_groups, err);
            continue;                  // an internal child groups its own children
        }
        if (!pack) {
            emit_group(cf, cc, sorder, body_slot, nbodies, groups, cap, n_groups, err);
            continue;
        }
        if (run_cnt + cc > kGroupMax) {
            emit_group(run_first, run_cnt, sorder, body_slot, nbodies, groups, cap, n_groups, err);
            run_first = -1;
            run_cnt = 0;
        }
        if (run_first < 0) run_first = cf;
        run_cnt += cc;
    }
    emit_group(run_first, run_cnt, sorder, body_slot, nbodies, groups, cap, n_groups, err);
}

// Interactions of one target (negated coordinates duplicated in both halves
// of n*) with TWO accepted cells at once (their values paired in the float2
// operands): monopole with the force law plus the Newtonian quadrupole term,
//   a += w x - Q x / r^5 + 5/2 (x.Q.x) x / r^7,  x = com - p,
// w the force law's (softened) monopole factor.  The list holds -Q (the q*
// arguments), which saves a negation per pair.  Under the reference law 1/r
// comes from the law's own reciprocal square root,
//   1/r = (r^2 + S) / sqrt(r^2 (r^2 + S)^2),
// one multiply instead of a second reciprocal square root.
template <int LAW>
__device__ __forceinline__ void cell_pair_accel(float2 cx, float2 cy, float2 cz, float2 cm, float2 qxx, float2 qyy,
                                                float2 qzz, float2 qxy, float2 qxz, float2 qyz, float2 nx, float2 ny,
                                                float2 nz, float2 S2, float2 T2, float2& ax, float2& ay, float2& az) {
    const float2 dx = __fadd2_rn(cx, nx);
    const float2 dy = __fadd2_rn(cy, ny);
    const float2 dz = __fadd2_rn(cz, nz);
    float2 r2 = __fmul2_rn(dx, dx);
    r2 = __ffma2_rn(dy, dy, r2);
    r2 = __ffma2_rn(dz, dz, r2);
    float2 w, ir;
    if (LAW == NB_LAW_REFERENCE) {
        const float2 s = __fadd2_rn(r2, S2);
        const float2 t = __ffma2_rn(__fmul2_rn(r2, s), s, T2);
        const float2 rt = make_float2(rsqrt_approx(t.x), rsqrt_approx(t.y));
        w = __fmul2_rn(cm, rt);
        ir = __fmul2_rn(rt, s);
    } else {
        const float2 q = __fadd2_rn(r2, S2);
        const float2 inv = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
        w = __fmul2_rn(__fmul2_rn(cm, inv), __fmul2_rn(inv, inv));
        ir = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
    }
    const float2 ir2 = __fmul2_rn(ir, ir);
    const float2 ir5 = __fmul2_rn(__fmul2_rn(ir2, ir), ir2);
    // q = -Q x, xqx = -x.Q.x
    const float2 qx = __ffma2_rn(qxx, dx, __ffma2_rn(qxy, dy, __fmul2_rn(qxz, dz)));
    const float2 qy = __ffma2_rn(qxy, dx, __ffma2_rn(qyy, dy, __fmul2_rn(qyz, dz)));
    const float2 qz = __ffma2_rn(qxz, dx, __ffma2_rn(qyz, dy, __fmul2_rn(qzz, dz)));
    const float2 xqx = __ffma2_rn(dx, qx, __ffma2_rn(dy, qy, __fmul2_rn(dz, qz)));
    const float2 c7 = __fmul2_rn(ir5, __fmul2_rn(ir2, make_float2(-2.5f, -2.5f)));
    const float2 wc = __ffma2_rn(xqx, c7, w);
    ax = __ffma2_rn(wc, dx, __ffma2_rn(ir5, qx, ax));
    ay = __ffma2_rn(wc, dy, __ffma2_rn(ir5, qy, ay));
    az = __ffma2_rn(wc, dz, __ffma2_rn(ir5, qz, az));
}

// Shared-memory lists hold their entries in pairs, each value of the two
// entries side by side, so that one 16-byte load yields two FP32x2 operands:
// a body pair is (x x' y y')(z z' m m'), a cell pair (x x' y y')(z z' m m')
// then -Q: (Qxx Qxx' Qyy Qyy')(Qzz Qzz' Qxy Qxy')(Qxz Qxz' Qyz Qyz'), negated.
constexpr float kFarAway = 1e18f;   // position of the zero-mass cell that pads an odd list

__device__ __forceinline__ void put_body(float4 (*lst)[2], int j, float4 b) {
    float* f = reinterpret_cast<float*>(lst[j >> 1]);
    const int h = j & 1;
    f[h] = b.x; f[2 + h] = b.y; f[4 + h] = b.z; f[6 + h] = b.w;
}

__device__ __forceinline__ void put_cell(float4 (*lst)[5], int j, float4 cm, float4 q1, float4 q2) {
    float* f = reinterpret_cast<float*>(lst[j >> 1]);
    const int h = j & 1;
    f[h] = cm.x; f[2 + h] = cm.y; f[4 + h] = cm.z; f[6 + h] = cm.w;
    f[8 + h] = -q1.x; f[10 + h] = -q1.y; f[12 + h] = -q1.z; f[14 + h] = -q2.x;
    f[16 + h] = -q2.y; f[18 + h] = -q2.z;
}

// Far field of a group: accepted cells that are far from the group compared
// with its size (group half-diagonal < eta * distance from the box centre X)
// act through a local expansion at X instead of once per body:
//   a(X + y) = A + J y + 1/2 H(y, y) + 1/6 T(y, y, y),
// A the cell's full acceleration at X (force law + quadrupole), J the first
// derivative of its Newtonian monopole + quadrupole field, H and T the second
// and third derivatives of the monopole field (with d = COM - X, r = |d|,
// s = d.Q.d):
//   J_ij   = m (3 d_i d_j / r^5 - delta_ij / r^3)
//          + Q_ij / r^5 - 5 ((Qd)_i d_j + (Qd)_j d_i) / r^7 - 5/2 s delta_ij / r^7 + 35/2 s d_i d_j / r^9,
//   H_ijk  = m (15 d_i d_j d_k / r^7 - 3 (delta_ik d_j + delta_jk d_i + delta_ij d_k) / r^5),
//   T_ijkl = m (105 d_i d_j d_k d_l / r^9 - 15 (delta_ij d_k d_l + 5 more pairings) / r^7
//               + 3 (delta_ij delta_kl + delta_ik delta_jl + delta_il delta_jk) / r^5)
// (the quadrupole part of J is minus the derivative, with respect to d, of
// the quadrupole acceleration -Q d / r^5 + 5/2 s d / r^7).  Each is a
// derivative tensor of a harmonic potential, so every trace vanishes and only
// the independent components are summed: J 5 (zz = -xx - yy), H 7 (xzz, yzz,
// zzz from the traces), T 9 (xxzz, yyzz, zzzz, xyzz, xzzz, yzzz from the
// traces).  The truncation error of a cell's term falls as (size / distance)^4.
constexpr int kFarTerms = 24;   // A (3), J xx yy xy xz yz (5), H (7), T (9)
struct FarField {
    float v[kFarTerms];
};

// Adds one cell's terms to a lane's partial sums (term k at f[k * stride]).
template <int LAW>
__device__ __forceinline__ void far_add(float* f, int stride, const float4 cm, const float4 q1, const float4 q2,
                                        float Xx, float Xy, float Xz, float S) {
    const float dx = cm.x - Xx, dy = cm.y - Xy, dz = cm.z - Xz;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float m = cm.w;
    float w;
    if (LAW == NB_LAW_REFERENCE) {
        const float s = r2 + S;
        w = m * rsqrt_approx(fmaf(r2 * s, s, kTiny));
    } else {
        const float inv = rsqrt_approx(r2 + S);
        w = m * inv * (inv * inv);
    }
    const float ir = rsqrt_approx(r2), ir2 = ir * ir, ir3 = ir2 * ir, ir5 = ir3 * ir2, ir7 = ir5 * ir2;
    // quadrupole term at X (Q traceless: q1 = Qxx Qyy Qzz, q2 = Qxy Qxz Qyz)
    const float qx = fmaf(q1.x, dx, fmaf(q2.x, dy, q2.y * dz));
    const float qy = fmaf(q2.x, dx, fmaf(q1.y, dy, q2.z * dz));
    const float qz = fmaf(q2.y, dx, fmaf(q2.z, dy, q1.z * dz));
    const float sq = fmaf(dx, qx, fmaf(dy, qy, dz * qz));   // d.Q.d
    const float c7 = 2.5f * sq * ir7;
    f[0 * stride] += fmaf(w + c7, dx, -qx * ir5);
    f[1 * stride] += fmaf(w + c7, dy, -qy * ir5);
    f[2 * stride] += fmaf(w + c7, dz, -qz * ir5);
    const float m3 = 3.f * m * ir5, m1 = m * ir3;
    const float t5 = 5.f * ir7, g9 = 17.5f * sq * ir7 * ir2, dg = m1 + c7;   // c7 = 5/2 s / r^7
    f[3 * stride] += fmaf(m3 * dx, dx, -dg) + fmaf(q1.x, ir5, dx * fmaf(g9, dx, -2.f * t5 * qx));   // J xx
    f[4 * stride] += fmaf(m3 * dy, dy, -dg) + fmaf(q1.y, ir5, dy * fmaf(g9, dy, -2.f * t5 * qy));   // J yy
    f[5 * stride] += fmaf(m3 * dx + g9 * dx, dy, fmaf(q2.x, ir5, -t5 * fmaf(qx, dy, qy * dx)));     // J xy
    f[6 * stride] += fmaf(m3 * dx + g9 * dx, dz, fmaf(q2.y, ir5, -t5 * fmaf(qx, dz, qz * dx)));     // J xz
    f[7 * stride] += fmaf(m3 * dy + g9 * dy, dz, fmaf(q2.z, ir5, -t5 * fmaf(qy, dz, qz * dy)));     // J yz
    const float m15 = 15.f * m * ir7;
    const float tx = m15 * dx, ty = m15 * dy;
    f[8 * stride] += dx * fmaf(tx, dx, -3.f * m3);    // H xxx = 15 m dx^3 / r^7 - 9 m dx / r^5
    f[9 * stride] += dy * fmaf(ty, dy, -3.f * m3);    // H yyy
    f[10 * stride] += dy * fmaf(tx, dx, -m3);         // H xxy
    f[11 * stride] += dz * fmaf(tx, dx, -m3);         // H xxz
    f[12 * stride] += dx * fmaf(ty, dy, -m3);         // H xyy
    f[13 * stride] += dz * fmaf(ty, dy, -m3);         // H yyz
    f[14 * stride] += tx * dy * dz;                   // H xyz
    const float a9 = 105.f * m * ir7 * ir2;           // 105 m / r^9
    const float x2 = dx * dx, y2 = dy * dy;
    const float ax2 = a9 * x2, ay2 = a9 * y2;
    f[15 * stride] += fmaf(x2, ax2 - 6.f * m15, 3.f * m3);          // T xxxx
    f[16 * stride] += fmaf(y2, ay2 - 6.f * m15, 3.f * m3);          // T yyyy
    f[17 * stride] += fmaf(ax2, y2, fmaf(-m15, x2 + y2, m3));        // T xxyy
    f[18 * stride] += dx * dy * (ax2 - 3.f * m15);                  // T xxxy
    f[19 * stride] += dx * dy * (ay2 - 3.f * m15);                  // T xyyy
    f[20 * stride] += dx * dz * (ax2 - 3.f * m15);                  // T xxxz
    f[21 * stride] += dx * dz * (ay2 - m15);                        // T xyyz
    f[22 * stride] += dy * dz * (ax2 - m15);                        // T xxyz
    f[23 * stride] += dy * dz * (ay2 - 3.f * m15);                  // T yyyz
}

// A + J y + 1/2 H(y, y) + 1/6 T(y, y, y) at offset y from the expansion centre.
__device__ __forceinline__ void far_eval(const FarField& f, float x, float y, float z, float& ax, float& ay,
                                         float& az) {
    const float* v = f.v;
    const float Jxx = v[3], Jyy = v[4], Jxy = v[5], Jxz = v[6], Jyz = v[7], Jzz = -Jxx - Jyy;
    const float Hxxx = v[8], Hyyy = v[9], Hxxy = v[10], Hxxz = v[11], Hxyy = v[12], Hyyz = v[13], Hxyz = v[14];
    const float Hxzz = -Hxxx - Hxyy, Hyzz = -Hxxy - Hyyy, Hzzz = -Hxxz - Hyyz;
    const float Txxxx = v[15], Tyyyy = v[16], Txxyy = v[17], Txxxy = v[18], Txyyy = v[19], Txxxz = v[20],
                Txyyz = v[21], Txxyz = v[22], Tyyyz = v[23];
    const float Txxzz = -Txxxx - Txxyy, Tyyzz = -Txxyy - Tyyyy, Tzzzz = -Txxzz - Tyyzz;
    const float Txyzz = -Txxxy - Txyyy, Txzzz = -Txxxz - Txyyz, Tyzzz = -Txxyz - Tyyyz;
    const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
    const float x3 = xx * x, y3 = yy * y, z3 = zz * z;
    const float x2y = xx * y, x2z = xx * z, xy2 = x * yy, y2z = yy * z, xz2 = x * zz, yz2 = y * zz, xyz = xy * z;
    constexpr float s6 = 1.f / 6.f;
    ax = v[0] + Jxx * x + Jxy * y + Jxz * z + 0.5f * (Hxxx * xx + Hxyy * yy + Hxzz * zz) + Hxxy * xy + Hxxz * xz +
         Hxyz * yz + s6 * (Txxxx * x3 + Txyyy * y3 + Txzzz * z3) +
         0.5f * (Txxxy * x2y + Txxxz * x2z + Txxyy * xy2 + Txxzz * xz2 + Txyyz * y2z + Txyzz * yz2) + Txxyz * xyz;
    ay = v[1] + Jxy * x + Jyy * y + Jyz * z + 0.5f * (Hxxy * xx + Hyyy * yy + Hyzz * zz) + Hxyy * xy + Hxyz * xz +
         Hyyz * yz + s6 * (Txxxy * x3 + Tyyyy * y3 + Tyzzz * z3) +
         0.5f * (Txxyy * x2y + Txxyz * x2z + Txyyy * xy2 + Txyzz * xz2 + Tyyyz * y2z + Tyyzz * yz2) + Txyyz * xyz;
    az = v[2] + Jxz * x + Jyz * y + Jzz * z + 0.5f * (Hxxz * xx + Hyyz * yy + Hzzz * zz) + Hxyz * xy + Hxzz * xz +
         Hyzz * yz + s6 * (Txxxz * x3 + Tyyyz * y3 + Tzzzz * z3) +
         0.5f * (Txxyz * x2y + Txxzz * x2z + Txyyz * xy2 + Txzzz * xz2 + Tyyzz * y2z + Tyzzz * yz2) + Txyzz * xyz;
}

// Persistent: each warp takes groups from the queue until it is empty.
template <int LAW>
__global__ void __launch_bounds__(kGWarps * 32, 5) k_group_traverse(
    const int4* __restrict__ groups, const int* __restrict__ n_groups_dev, int group_cap, int* __restrict__ next_group,
    const float4* __restrict__ spos, const int32_t* __restrict__ sorder, const CellRec* __restrict__ rec,
    const float4* __restrict__ gal_box, const int32_t* __restrict__ gal_root, int nslot, int n_cells, int nbodies,
    int max_pops, int leaf_size, float theta2, float S, float G, float far2, float far_rel, float far_cap2,
    float far_min_r2,
    const unsigned* __restrict__ mmax, float4* __restrict__ acc,
    unsigned long long* __restrict__ inter, int* __restrict__ err) {
    __shared__ int stk[kGWarps][kGStack];
    __shared__ float4 lcl[kGWarps][kGCells / 2][5];
    __shared__ float4 lbd[kGWarps][kGBodies / 2][2];
    __shared__ float ffs[kGWarps][kFarTerms][32];   // far-field partial sums, one column per lane
    __shared__ int rinc[kGWarps][32], rfst[kGWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const int ngroups = min(*n_groups_dev, group_cap);
    const float2 S2 = make_float2(S, S);
    const float tiny = self_pair_tiny(mmax);   // a leaf's bodies include the target itself
    const float2 T2 = make_float2(tiny, tiny);
    unsigned long long total = 0;
    for (;;) {
    int gi = 0;
    if (lane == 0) gi = atomicAdd(next_group, 1);
    gi = __shfl_sync(0xffffffffu, gi, 0);
    if (gi >= ngroups) break;
    const int4 grp = groups[gi];   // (slot, first sorted position, count, 0)
    if (grp.x < 0 || grp.x >= nslot || grp.y < 0 || grp.z < 1 || grp.z > kGroupMax || grp.y + grp.z > nbodies) {
        if (lane == 0) record_error(err, DEV_TREE_OVERFLOW);
        continue;
    }
    const bool v0 = lane < grp.z, v1 = lane + 32 < grp.z;
    const bool dual = grp.z > 32;   // warp-uniform: groups of at most 32 bodies evaluate one body per lane
    const int s0 = grp.y + (v0 ? lane : 0), s1 = grp.y + (v1 ? lane + 32 : 0);
    const float4 p0 = spos[s0], p1 = spos[s1];
    float bl[3], bh[3];
    {
        const float a0[3] = {p0.x, p0.y, p0.z}, a1[3] = {p1.x, p1.y, p1.z};
        for (int a = 0; a < 3; ++a) {
            bl[a] = fminf(v0 ? a0[a] : INFINITY, v1 ? a1[a] : INFINITY);
            bh[a] = fmaxf(v0 ? a0[a] : -INFINITY, v1 ? a1[a] : -INFINITY);
            for (int o = 16; o > 0; o >>= 1) {
                bl[a] = fminf(bl[a], __shfl_xor_sync(0xffffffffu, bl[a], o));
                bh[a] = fmaxf(bh[a], __shfl_xor_sync(0xffffffffu, bh[a], o));
            }
        }
    }
    const float4 gb = gal_box[grp.x];
    // expansion centre of the group's far field and its half-diagonal squared
    const float Xx = 0.5f * (bl[0] + bh[0]), Xy = 0.5f * (bl[1] + bh[1]), Xz = 0.5f * (bl[2] + bh[2]);
    const float rg2 = 0.25f * ((bh[0] - bl[0]) * (bh[0] - bl[0]) + (bh[1] - bl[1]) * (bh[1] - bl[1]) +
                               (bh[2] - bl[2]) * (bh[2] - bl[2]));
    // relative far-field rule: the group's smallest |a| / G of the previous
    // evaluation (none yet: 0, the geometric rule decides)
    float far_thr = 0.f;
    if (far_rel > 0.f) {
        float a2 = INFINITY;
        if (v0) {
            const float4 a = acc[sorder[s0]];
            a2 = fmaf(a.z, a.z, fmaf(a.y, a.y, a.x * a.x));
        }
        if (v1) {
            const float4 a = acc[sorder[s1]];
            a2 = fminf(a2, fmaf(a.z, a.z, fmaf(a.y, a.y, a.x * a.x)));
        }
        for (int o = 16; o > 0; o >>= 1) a2 = fminf(a2, __shfl_xor_sync(0xffffffffu, a2, o));
        if (a2 > 0.f && a2 < INFINITY) far_thr = far_rel * sqrtf(a2);
    }
    const bool use_far = far2 > 0.f || far_rel > 0.f;
    for (int k = 0; k < kFarTerms; ++k) ffs[w][k][lane] = 0.f;   // this lane's share of the far field
    // negated target coordinates, duplicated: the pair partner is the other list entry
    const float2 n0x = make_float2(-p0.x, -p0.x), n0y = make_float2(-p0.y, -p0.y), n0z = make_float2(-p0.z, -p0.z);
    const float2 n1x = make_float2(-p1.x, -p1.x), n1y = make_float2(-p1.y, -p1.y), n1z = make_float2(-p1.z, -p1.z);
    const float2 z2 = make_float2(0.f, 0.f);
    float2 a0x = z2, a0y = z2, a0z = z2, a1x = z2, a1y = z2, a1z = z2;   // (even entries, odd entries)
    float s0x = 0.f, s0y = 0.f, s0z = 0.f, c0x = 0.f, c0y = 0.f, c0z = 0.f;
    float s1x = 0.f, s1y = 0.f, s1z = 0.f, c1x = 0.f, c1y = 0.f, c1z = 0.f;
    unsigned cnt = 0;
    const unsigned nv = (v0 ? 1u : 0u) + (v1 ? 1u : 0u);
    int nst = 0, ncl = 0, nbd = 0, pops = 0;
    bool bad = false;

    auto fold = [&]() {
        kahan_add(s0x, c0x, a0x.x + a0x.y); kahan_add(s0y, c0y, a0y.x + a0y.y); kahan_add(s0z, c0z, a0z.x + a0z.y);
        kahan_add(s1x, c1x, a1x.x + a1x.y); kahan_add(s1y, c1y, a1y.x + a1y.y); kahan_add(s1z, c1z, a1z.x + a1z.y);
        a0x = a0y = a0z = a1x = a1y = a1z = z2;
    };
    auto flush_cells = [&]() {
        if (ncl & 1) {   // pad with a zero-mass, zero-moment cell far away: adds exactly zero
            if (lane == 0)
                put_cell(lcl[w], ncl, make_float4(kFarAway, kFarAway, kFarAway, 0.f), make_float4(0.f, 0.f, 0.f, 0.f),
                         make_float4(0.f, 0.f, 0.f, 0.f));
        }
        __syncwarp();
        auto cell_loop = [&](auto both) {
            for (int k = 0; k < (ncl + 1) >> 1; ++k) {
                const float4 e0 = lcl[w][k][0], e1 = lcl[w][k][1], e2 = lcl[w][k][2], e3 = lcl[w][k][3],
                             e4 = lcl[w][k][4];
                const float2 cx = make_float2(e0.x, e0.y), cy = make_float2(e0.z, e0.w), cz = make_float2(e1.x, e1.y);
                const float2 cm = make_float2(e1.z, e1.w), qxx = make_float2(e2.x, e2.y), qyy = make_float2(e2.z, e2.w);
                const float2 qzz = make_float2(e3.x, e3.y), qxy = make_float2(e3.z, e3.w), qxz = make_float2(e4.x, e4.y);
                const float2 qyz = make_float2(e4.z, e4.w);
                cell_pair_accel<LAW>(cx, cy, cz, cm, qxx, qyy, qzz, qxy, qxz, qyz, n0x, n0y, n0z, S2, T2, a0x, a0y,
                                     a0z);
                if (decltype(both)::value)
                    cell_pair_accel<LAW>(cx, cy, cz, cm, qxx, qyy, qzz, qxy, qxz, qyz, n1x, n1y, n1z, S2, T2, a1x, a1y,
                                         a1z);
            }
        };
        if (dual) cell_loop(std::true_type{}); else cell_loop(std::false_type{});
        cnt += nv * ncl;
        ncl = 0;
        fold();
        __syncwarp();
    };
    auto flush_bodies = [&]() {
        if (nbd & 1) {   // pad with a zero-mass body: adds exactly zero
            if (lane == 0) put_body(lbd[w], nbd, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        __syncwarp();
        const int np = (nbd + 1) >> 1;
        auto body_loop = [&](auto both) {
            int k = 0;
#pragma unroll 1
            for (; k + 2 <= np; k += 2) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float4 e0 = lbd[w][k + u][0], e1 = lbd[w][k + u][1];
                    const float2 bx = make_float2(e0.x, e0.y), by = make_float2(e0.z, e0.w);
                    const float2 bz = make_float2(e1.x, e1.y), bm = make_float2(e1.z, e1.w);
                    interact_x2<LAW>(bx, by, bz, bm, n0x, n0y, n0z, S2, T2, a0x, a0y, a0z);
                    if (decltype(both)::value)
                        interact_x2<LAW>(bx, by, bz, bm, n1x, n1y, n1z, S2, T2, a1x, a1y, a1z);
                }
            }
            for (; k < np; ++k) {
                const float4 e0 = lbd[w][k][0], e1 = lbd[w][k][1];
                const float2 bx = make_float2(e0.x, e0.y), by = make_float2(e0.z, e0.w);
                const float2 bz = make_float2(e1.x, e1.y), bm = make_float2(e1.z, e1.w);
                interact_x2<LAW>(bx, by, bz, bm, n0x, n0y, n0z, S2, T2, a0x, a0y, a0z);
                if (decltype(both)::value) interact_x2<LAW>(bx, by, bz, bm, n1x, n1y, n1z, S2, T2, a1x, a1y, a1z);
            }
        };
        if (dual) body_loop(std::true_type{}); else body_loop(std::false_type{});
        cnt += nv * nbd;
        nbd = 0;
        fold();
        __syncwarp();
    };
    // Appends the bodies of this step's accepted leaf ranges (lane l: first,
    // count; count 0 for lanes without one) to the body list, all lanes
    // copying, evaluating the list whenever it fills.
    auto gather_ranges = [&](int first, int count) {
        int incl = count;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int tot = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        rinc[w][lane] = incl;
        rfst[w][lane] = first;
        __syncwarp();
        for (int done = 0; done < tot;) {
            if (nbd == kGBodies) flush_bodies();
            const int take = min(kGBodies - nbd, tot - done);
            for (int j = lane; j < take; j += 32) {
                const int jj = done + j;
                int lo = 0, hi = 31;   // owner: the first lane whose inclusive end exceeds jj
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (rinc[w][mid] > jj) hi = mid; else lo = mid + 1;
                }
                const int base = lo > 0 ? rinc[w][lo - 1] : 0;
                put_body(lbd[w], nbd + j, spos[rfst[w][lo] + (jj - base)]);
            }
            nbd += take;
            done += take;
            __syncwarp();
        }
    };

    const int root = gal_root[grp.x];
    if (root < 1 || root >= n_cells) {
        bad = true;
    } else {
        const int4 rw = __ldg(&rec[root].walk);
        const int rF = rw.x, rn = (rw.w >> 4) & 15;
        if ((rw.w & 15) != BK_INTERNAL || rF < 1 || rn < 1 || rn > 8 || rF + rn > n_cells || rF >= kStackCellLimit) {
            bad = true;
        } else {
            if (lane == 0) stk[w][0] = (rF << 4) | rn;
            nst = 1;
        }
    }
    __syncwarp();
    while (nst > 0 && !bad) {
        if (++pops > max_pops) { bad = true; break; }
        // Take up to 8 opened cells from the top of the stack, as many as have
        // at most 32 children together; lane j tests the j-th of those children.
        // Above kGMultiTop waiting cells a step takes one cell (a depth-first
        // walk leaving at most 7 cells per level, 7 * 21 + 8 in all), so the
        // stack stays below kGMultiTop + 31 + 155 < kGStack.
        const int cap = nst <= kGMultiTop ? 8 : 1;
        int pF = 0, pn = 0;
        if (lane < cap && lane < nst) {   // a stack entry is an opened cell's (first child << 4 | children)
            const int e = stk[w][nst - 1 - lane];
            pF = e >> 4;
            pn = e & 15;
        }
        int incl = pn;   // inclusive prefix of the child counts over lanes 0..7
        for (int o = 1; o < 8; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const uint32_t take = __ballot_sync(0xffffffffu, lane < cap && lane < nst && incl <= 32);
        const int P = __popc(take);   // >= 1: one cell has at most 8 children
        const int T = __shfl_sync(0xffffffffu, incl, P - 1);
        __syncwarp();
        nst -= P;
        // source cell of this lane's child: the last taken cell starting at or
        // before it (every opened cell has at least one child, so the starts differ)
        const uint32_t starts = __reduce_or_sync(0xffffffffu, lane < P ? 1u << (incl - pn) : 0u);
        const int q = __popc(starts & ((2u << lane) - 1u)) - 1;
        const int qF = __shfl_sync(0xffffffffu, pF, q & 7);
        const int qx = __shfl_sync(0xffffffffu, incl - pn, q & 7);
        bool a_cell = false, a_range = false, a_push = false, a_bad = false;
        float4 ccm = make_float4(0.f, 0.f, 0.f, 0.f);
        int first = 0, count = 0, ch = 0, cF = 0, cn = 0;
        if (lane < T) {
            ch = qF + (lane - qx);
            ccm = __ldg(&rec[ch].com);
            const int4 wr = __ldg(&rec[ch].walk);
            const int kind = wr.w & 15;
            count = wr.y;
            first = wr.z;
            cF = wr.x;
            cn = (wr.w >> 4) & 15;
            // The group form of the reference's rule side / r < theta: r is bounded
            // below for every body of the group by the distance from the centre of
            // mass to the group's bounding box.
            const float side = ldexpf(gb.w, kSlotLevels - (wr.w >> 8));
            float d2 = 0.f;
            const float cc[3] = {ccm.x, ccm.y, ccm.z};
            for (int a = 0; a < 3; ++a) {
                const float d = fmaxf(0.f, fmaxf(bl[a] - cc[a], cc[a] - bh[a]));
                d2 = fmaf(d, d, d2);
            }
            const bool accept = side * side < theta2 * d2;
            a_cell = accept && count > 2 && kind == BK_INTERNAL;
            a_range = !a_cell && (count <= leaf_size || kind != BK_INTERNAL);
            a_push = !a_cell && !a_range;
            if (a_cell && use_far) {
                const float ex = ccm.x - Xx, ey = ccm.y - Xy, ez = ccm.z - Xz;
                const float r2X = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                bool far;
                if (far_thr > 0.f) {   // m / r^2 (r_g / r)^4 < alpha |a|_min / G, r_g / r < cap
                    const float q = rg2 / r2X;
                    far = rg2 < far_cap2 * r2X && ccm.w * q * q < far_thr * r2X;
                } else {
                    far = rg2 < far2 * r2X;
                }
                if (far && r2X > far_min_r2) {   // far: into the group's local expansion
                    far_add<LAW>(&ffs[w][0][lane], 32, ccm, __ldg(&rec[ch].q1), __ldg(&rec[ch].q2), Xx, Xy, Xz, S);
                    cnt += (unsigned)grp.z;
                    a_cell = false;   // accepted, not listed
                }
            }
            // node data outside the body range would be a corrupt tree: report, never dereference
            if (a_range && (first < 0 || count < 0 || first + count > nbodies)) a_range = false, a_bad = true;
            if (a_push && (cF < 1 || cn < 1 || cn > 8 || cF + cn > n_cells || cF >= kStackCellLimit))
                a_push = false, a_bad = true;
        }
        if (__any_sync(0xffffffffu, a_bad)) { bad = true; break; }
        const uint32_t bc = __ballot_sync(0xffffffffu, a_cell);
        if (bc) {
            if (ncl + __popc(bc) > kGCells) flush_cells();
            if (a_cell) {
                const int idx = ncl + __popc(bc & lt);
                put_cell(lcl[w], idx, ccm, __ldg(&rec[ch].q1), __ldg(&rec[ch].q2));
            }
            ncl += __popc(bc);
        }
        const uint32_t br = __ballot_sync(0xffffffffu, a_range);
        if (br) gather_ranges(a_range ? first : 0, a_range ? count : 0);
        const uint32_t bp = __ballot_sync(0xffffffffu, a_push);
        if (bp) {
            if (nst + __popc(bp) > kGStack) { bad = true; break; }
            if (a_push) stk[w][nst + __popc(bp & lt)] = (cF << 4) | cn;
            nst += __popc(bp);
        }
        __syncwarp();
    }
    if (!bad) {
        flush_cells();
        flush_bodies();
    }
    fold();
    // the group's far field: sum the lanes' partial expansions, evaluate at each body
    if (use_far) {
        FarField ff;
        for (int k = 0; k < kFarTerms; ++k) {
            float x = ffs[w][k][lane];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            ff.v[k] = x;
        }
        float fx, fy, fz;
        far_eval(ff, p0.x - Xx, p0.y - Xy, p0.z - Xz, fx, fy, fz);
        kahan_add(s0x, c0x, fx); kahan_add(s0y, c0y, fy); kahan_add(s0z, c0z, fz);
        far_eval(ff, p1.x - Xx, p1.y - Xy, p1.z - Xz, fx, fy, fz);
        kahan_add(s1x, c1x, fx); kahan_add(s1y, c1y, fy); kahan_add(s1z, c1z, fz);
    }
    if (bad && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
    if (v0) acc[sorder[s0]] = make_float4(G * (s0x - c0x), G * (s0y - c0y), G * (s0z - c0z), 0.f);
    if (v1) acc[sorder[s1]] = make_float4(G * (s1x - c1x), G * (s1y - c1y), G * (s1z - c1z), 0.f);
    total += cnt;
    }
    for (int o = 16; o > 0; o >>= 1) total += __shfl_down_sync(0xffffffffu, total, o);
    if (lane == 0 && total) atomicAdd(inter, total);
}

// ---- batched direct sum --------------------------------------------------------
// unit = (first target body, first source tile, source tiles, index of the
// target's sum partial); the compensation partial follows at +comp_offset of
// the unit's galaxy, kept in unit_comp.
template <int LAW, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK) k_batch_direct(const float4* __restrict__ pos, const int4* __restrict__ units,
                                                        const int32_t* __restrict__ unit_comp, int nunits,
                                                        int* __restrict__ next_unit, float S,
                                                        const unsigned* __restrict__ mmax,
                                                        float4* __restrict__ part) {
    __shared__ float4 tile[kDirTile];
    const float tiny = self_pair_tiny(mmax);
    __shared__ int cur;
    static_assert(kDirTile % BLOCK == 0 || BLOCK % kDirTile == 0, "tile/block");
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) cur = atomicAdd(next_unit, 1);
        __syncthreads();
        const int u = cur;
        if (u >= nunits) return;
        const int4 un = units[u];
        float xi[IPT], yi[IPT], zi[IPT], sx[IPT], sy[IPT], sz[IPT], cx[IPT], cy[IPT], cz[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const float4 q = pos[un.x + k * BLOCK + threadIdx.x];
            xi[k] = q.x; yi[k] = q.y; zi[k] = q.z;
            sx[k] = sy[k] = sz[k] = cx[k] = cy[k] = cz[k] = 0.f;
        }
        for (int t = 0; t < un.z; ++t) {
            __syncthreads();
            for (int j = threadIdx.x; j < kDirTile; j += BLOCK) tile[j] = pos[(size_t)(un.y + t) * kDirTile + j];
            __syncthreads();
#pragma unroll 1
            for (int f = 0; f < kDirTile; f += kFold) {
                float tx[IPT], ty[IPT], tz[IPT];
#pragma unroll
                for (int k = 0; k < IPT; ++k) tx[k] = ty[k] = tz[k] = 0.f;
#pragma unroll 4
                for (int j = 0; j < kFold; ++j) {
                    const float4 pj = tile[f + j];
#pragma unroll
                    for (int k = 0; k < IPT; ++k)
                        interact<LAW>(pj, xi[k], yi[k], zi[k], S, tiny, tx[k], ty[k], tz[k]);
                }
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    kahan_add(sx[k], cx[k], tx[k]);
                    kahan_add(sy[k], cy[k], ty[k]);
                    kahan_add(sz[k], cz[k], tz[k]);
                }
            }
        }
        const int co = unit_comp[u];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int d = k * BLOCK + threadIdx.x;
            part[(size_t)un.w + d] = make_float4(sx[k], sy[k], sz[k], 0.f);
            part[(size_t)un.w + co + d] = make_float4(cx[k], cy[k], cz[k], 0.f);
        }
    }
}

// folds the partials of direct-sum body i (global index begin + i) into acc.
__global__ void k_batch_direct_reduce(const int32_t* __restrict__ body_dgal, const int4* __restrict__ dgal /* off, n_pad, splits, part_base */,
                                      int begin, int count, float G, const float4* __restrict__ part,
                                      float4* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int g = body_dgal[i];
    if (g < 0) return;   // padding body
    const int4 d = dgal[g];
    const int local = begin + i - d.x;
    float ax = 0.f, ay = 0.f, az = 0.f, kx = 0.f, ky = 0.f, kz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
    for (int s = 0; s < d.z; ++s) {
        const float4 p = part[(size_t)d.w + (size_t)s * d.y + local];
        const float4 c = part[(size_t)d.w + (size_t)(d.z + s) * d.y + local];
        kahan_add(ax, kx, p.x);
        kahan_add(ay, ky, p.y);
        kahan_add(az, kz, p.z);
        qx += c.x; qy += c.y; qz += c.z;
    }
    acc[begin + i] = make_float4(G * (ax - (kx + qx)), G * (ay - (ky + qy)), G * (az - (kz + qz)), 0.f);
}

}  // namespace nb
