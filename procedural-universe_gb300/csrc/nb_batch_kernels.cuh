// nb_batch_kernels.cuh -- kernels of the batched form (included by nb_batch.cu).
//
// Many independent galaxies are stepped together, one launch per phase:
//  * Barnes-Hut members (n >= threshold) are stored first, contiguously.  Each
//    gets a tight bounding cube; a body's key is its galaxy slot (21 bits, the
//    top 7 octal levels) followed by a 42-bit Morton code in its cube (14
//    levels), so ONE radix sort and ONE topology build make a forest whose
//    level-7 nodes are the galaxy roots.
//  * The mass pass adds traceless quadrupole moments (parallel-axis rule
//    bottom-up), and the traversal is group-wise: a warp takes up to 32
//    consecutive sorted bodies of one galaxy, opens a cell when the cell
//    side exceeds theta times the distance from the cell's centre of mass to
//    the group's bounding box, and collects accepted cells (monopole +
//    quadrupole) and leaf buckets of at most leaf_size bodies (summed body by
//    body) in shared-memory lists that every lane then evaluates -- no lane
//    idles on a per-lane decision.  This is a performance form whose parity
//    is the force error against the FP64 direct sum (<= 1e-3), not the
//    reference's per-body opening rule.
//  * Direct-sum members are padded to multiples of 256 bodies; a persistent
//    kernel takes (galaxy, target block, source range) units from a table
//    through an atomic counter, and a second kernel folds the partials.
#pragma once

namespace nb {

constexpr int kSlotLevels = 7;          // 21 bits of galaxy slot
constexpr int kMortonLevels = 14;       // 42 bits of position in the galaxy cube
constexpr int kBatchDepth = kSlotLevels + kMortonLevels;
constexpr int kGWarps = 4;              // warps per traversal block
constexpr int kGStack = 128;            // cells waiting to be opened, per warp
constexpr int kGCells = 64;             // accepted-cell list, per warp
constexpr int kGRanges = 32;            // leaf-bucket list, per warp
constexpr int kDirTile = 128;           // sources per shared tile of the batched direct kernel

enum : int { BK_SINGLE = 1, BK_BUCKET = 2, BK_INTERNAL = 3 };

// ---- bounding cube of each Barnes-Hut galaxy (one block per galaxy) -------
__global__ void k_gal_box(const float4* __restrict__ pos, const int4* __restrict__ gal /* off, n */, int ngal,
                          float4* __restrict__ box) {
    const int g = blockIdx.x;
    if (g >= ngal) return;
    const int4 gi = gal[g];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < gi.y; i += blockDim.x) {
        const float4 p = pos[gi.x + i];
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
    __shared__ float sh[6][32];
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { sh[a][w] = lo[a]; sh[3 + a][w] = hi[a]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; ++k)
            for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], sh[a][k]); hi[a] = fmaxf(hi[a], sh[3 + a][k]); }
        float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
        ext = fmaxf(ext * 1.001f, 1e-20f);
        box[g] = make_float4(lo[0], lo[1], lo[2], ext);
    }
}

__device__ __forceinline__ uint64_t spread3(uint32_t v) {   // 14 bits -> every third bit
    uint64_t x = v & 0x3fffu;
    x = (x | (x << 16)) & 0x0000ff0000ffull;
    x = (x | (x << 8)) & 0x00f00f00f00full;
    x = (x | (x << 4)) & 0x0c30c30c30c3ull;
    x = (x | (x << 2)) & 0x249249249249ull;
    return x;
}

// keys of Barnes-Hut bodies [0, n); pad entries [n, nk) get key ~0.
__global__ void k_batch_keys(const float4* __restrict__ pos, const int32_t* __restrict__ body_slot, int n, int nk,
                             const float4* __restrict__ box, uint64_t* __restrict__ keys, int32_t* __restrict__ vals,
                             int32_t* __restrict__ depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nk) return;
    vals[i] = i;
    if (i >= n) {
        keys[i] = ~0ull;
        return;
    }
    const int slot = body_slot[i];
    const float4 b = box[slot];
    const float4 p = pos[i];
    const float sc = 16384.0f / b.w;
    const uint32_t qx = (uint32_t)min(max((p.x - b.x) * sc, 0.f), 16383.f);
    const uint32_t qy = (uint32_t)min(max((p.y - b.y) * sc, 0.f), 16383.f);
    const uint32_t qz = (uint32_t)min(max((p.z - b.z) * sc, 0.f), 16383.f);
    keys[i] = ((uint64_t)slot << (3 * kMortonLevels)) | spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
    depth[i] = kBatchDepth;
}

// ---- bottom-up mass, centre of mass and quadrupole --------------------------
// Q_ij = sum m (3 y_i y_j - |y|^2 d_ij), y = offset from the node's centre of
// mass; a parent sums its children's Q plus m_c (3 d d - |d|^2 I), d = com_c - com.
__device__ void bucket_moments(const float4* spos, int first, int count, float4& cm, float4& q1, float4& q2) {
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

__device__ void finish_moments(int k, const int32_t* int_cell, const int32_t* int_block, const uint32_t* int_mask,
                               const int32_t* int_first, const float4* spos, float4* cell_com, float4* cell_q1,
                               float4* cell_q2, int32_t* cell_count, int32_t* cell_first, const int4* cell_meta,
                               int cell_cap, int nbodies, int* err) {
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
        const int ch = F + j;
        const int4 mt = __ldcg(&cell_meta[ch]);
        const int kind = mt.w & 15;
        const int cnt = __ldcg(&cell_count[ch]);
        if (kind == BK_INTERNAL) {
            ccm[j] = __ldcg(&cell_com[ch]);
            cq1[j] = __ldcg(&cell_q1[ch]);
            cq2[j] = __ldcg(&cell_q2[ch]);
        } else if (kind == BK_BUCKET) {
            if (mt.x < 0 || cnt < 0 || mt.x + cnt > nbodies) {
                record_error(err, DEV_TREE_OVERFLOW);
                ccm[j] = cq1[j] = cq2[j] = make_float4(0.f, 0.f, 0.f, 0.f);
                continue;
            }
            bucket_moments(spos, mt.x, cnt, ccm[j], cq1[j], cq2[j]);
        } else {
            ccm[j] = __ldcg(&cell_com[ch]);
            cq1[j] = cq2[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        m += ccm[j].w;
        cx = fmaf(ccm[j].w, ccm[j].x, cx); cy = fmaf(ccm[j].w, ccm[j].y, cy); cz = fmaf(ccm[j].w, ccm[j].z, cz);
        count += cnt;
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
    __stcg(&cell_com[c], make_float4(cx, cy, cz, m));
    __stcg(&cell_q1[c], make_float4(xx, yy, zz, 0.f));
    __stcg(&cell_q2[c], make_float4(xy, xz, yz, 0.f));
    __stcg(&cell_count[c], count);
    __stcg(&cell_first[c], int_first[k]);
}

__global__ void k_batch_moments(int int_cap, const int32_t* __restrict__ n_int_dev,
                                const int32_t* __restrict__ int_parent, const int32_t* __restrict__ int_nint,
                                int32_t* __restrict__ int_pending, const int32_t* __restrict__ int_cell,
                                const int32_t* __restrict__ int_block, const uint32_t* __restrict__ int_mask,
                                const int32_t* __restrict__ int_first, const float4* __restrict__ spos,
                                float4* __restrict__ cell_com, float4* __restrict__ cell_q1,
                                float4* __restrict__ cell_q2, int32_t* __restrict__ cell_count,
                                int32_t* __restrict__ cell_first, const int4* __restrict__ cell_meta, int cell_cap,
                                int nbodies, int* __restrict__ err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int ni = min(*n_int_dev, int_cap);
    if (k >= ni || int_nint[k] != 0) return;
    for (int guard = 0; guard < 64; ++guard) {
        finish_moments(k, int_cell, int_block, int_mask, int_first, spos, cell_com, cell_q1, cell_q2, cell_count,
                       cell_first, cell_meta, cell_cap, nbodies, err);
        if (k == 0) return;
        __threadfence();
        const int p = int_parent[k];
        if (p < 0 || p >= ni) return;
        const int old = atomicAdd(&int_pending[p], 1);
        if (old != int_nint[p] - 1) return;
        __threadfence();
        k = p;
    }
}

// Root cell of each galaxy: the level-7 internal node starting at the
// galaxy's first sorted position.
__global__ void k_batch_roots(const int32_t* __restrict__ slot_start, int nslot, const uint64_t* __restrict__ keys,
                              const int32_t* __restrict__ int_base, const int32_t* __restrict__ int_cell,
                              const int32_t* __restrict__ n_int_dev, int int_cap, int32_t* __restrict__ root,
                              int32_t* __restrict__ err) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nslot) return;
    const int s = slot_start[g];
    int prev = -1;
    if (s > 0) {
        const uint64_t x = keys[s - 1] ^ keys[s];
        prev = x == 0 ? kBatchDepth : (__clzll((long long)x) - (64 - 3 * kBatchDepth)) / 3;
    }
    const int k = int_base[s] + (kSlotLevels - (prev + 1));
    if (prev + 1 > kSlotLevels || k < 0 || k >= min(*n_int_dev, int_cap)) {
        root[g] = -1;
        record_error(err, DEV_TREE_OVERFLOW);
        return;
    }
    root[g] = int_cell[k];
}

// ---- group traversal ----------------------------------------------------------
template <int LAW>
__device__ __forceinline__ void body_accel(const float4 p, const float4 b, float S, float& ax, float& ay, float& az) {
    const float dx = b.x - p.x, dy = b.y - p.y, dz = b.z - p.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    float w;
    if (LAW == NB_LAW_REFERENCE) {
        const float s = r2 + S;
        w = b.w * rsqrt_approx(fmaf(r2 * s, s, 1e-30f));
    } else {
        const float inv = rsqrt_approx(r2 + S);
        w = b.w * inv * (inv * inv);
    }
    ax = fmaf(w, dx, ax);
    ay = fmaf(w, dy, ay);
    az = fmaf(w, dz, az);
}

// Monopole with the force law plus the Newtonian quadrupole term
// a += Q x / r^5 - 5/2 (x.Q.x) x / r^7, x = p - com.
template <int LAW>
__device__ __forceinline__ void cell_accel(const float4 p, const float4 cm, const float4 q1, const float4 q2, float S,
                                           float& ax, float& ay, float& az) {
    const float dx = cm.x - p.x, dy = cm.y - p.y, dz = cm.z - p.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    float w;
    if (LAW == NB_LAW_REFERENCE) {
        const float s = r2 + S;
        w = cm.w * rsqrt_approx(fmaf(r2 * s, s, 1e-30f));
    } else {
        const float inv = rsqrt_approx(r2 + S);
        w = cm.w * inv * (inv * inv);
    }
    const float ir = rsqrt_approx(r2);
    const float ir2 = ir * ir;
    const float ir5 = ir2 * ir2 * ir;
    const float qx = fmaf(q1.x, dx, fmaf(q2.x, dy, q2.y * dz));
    const float qy = fmaf(q2.x, dx, fmaf(q1.y, dy, q2.z * dz));
    const float qz = fmaf(q2.y, dx, fmaf(q2.z, dy, q1.z * dz));
    const float c = 2.5f * fmaf(dx, qx, fmaf(dy, qy, dz * qz)) * ir5 * ir2;
    ax += fmaf(w + c, dx, -qx * ir5);
    ay += fmaf(w + c, dy, -qy * ir5);
    az += fmaf(w + c, dz, -qz * ir5);
}

template <int LAW>
__global__ void __launch_bounds__(kGWarps * 32) k_group_traverse(
    const int4* __restrict__ warps, int nwarps, const float4* __restrict__ spos, const int32_t* __restrict__ sorder,
    const float4* __restrict__ cell_com, const int4* __restrict__ cell_meta, const float4* __restrict__ cell_q1,
    const float4* __restrict__ cell_q2, const int32_t* __restrict__ cell_first, const int32_t* __restrict__ cell_count,
    const float4* __restrict__ cell_hi, const float4* __restrict__ gal_box, const int32_t* __restrict__ gal_root,
    int n_cells, int nbodies, int max_pops, int leaf_size, float theta2, float S, float G, float4* __restrict__ acc,
    unsigned long long* __restrict__ inter, int* __restrict__ err) {
    __shared__ int stk[kGWarps][kGStack];
    __shared__ float4 lcm[kGWarps][kGCells], lq1[kGWarps][kGCells], lq2[kGWarps][kGCells];
    __shared__ int2 lrg[kGWarps][kGRanges];
    __shared__ float4 bbuf[kGWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kGWarps + w;
    if (gw >= nwarps) return;   // whole warp
    const int4 wi = warps[gw];  // (slot, first sorted position, count, 0)
    const bool valid = lane < wi.z;
    const int s = wi.y + (valid ? lane : 0);
    const float4 p = spos[s];
    float bl[3] = {valid ? p.x : INFINITY, valid ? p.y : INFINITY, valid ? p.z : INFINITY};
    float bh[3] = {valid ? p.x : -INFINITY, valid ? p.y : -INFINITY, valid ? p.z : -INFINITY};
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            bl[a] = fminf(bl[a], __shfl_xor_sync(0xffffffffu, bl[a], o));
            bh[a] = fmaxf(bh[a], __shfl_xor_sync(0xffffffffu, bh[a], o));
        }
    const float4 gb = gal_box[wi.x];
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, tx = 0.f, ty = 0.f, tz = 0.f;
    unsigned cnt = 0;
    int nst = 0, ncl = 0, nrg = 0, pops = 0;
    bool bad = false;
    const uint32_t lt = (1u << lane) - 1u;

    auto flush_cells = [&]() {
        __syncwarp();
        for (int i = 0; i < ncl; ++i) cell_accel<LAW>(p, lcm[w][i], lq1[w][i], lq2[w][i], S, tx, ty, tz);
        cnt += valid ? ncl : 0;
        ncl = 0;
        kahan_add(sx, cx, tx); kahan_add(sy, cy, ty); kahan_add(sz, cz, tz);
        tx = ty = tz = 0.f;
        __syncwarp();
    };
    auto flush_ranges = [&]() {
        __syncwarp();
        for (int r = 0; r < nrg; ++r) {
            const int2 rg = lrg[w][r];
            for (int b0 = 0; b0 < rg.y; b0 += 32) {
                const int m = min(32, rg.y - b0);
                if (lane < m) bbuf[w][lane] = spos[rg.x + b0 + lane];
                __syncwarp();
                for (int j = 0; j < m; ++j) body_accel<LAW>(p, bbuf[w][j], S, tx, ty, tz);
                cnt += valid ? m : 0;
                __syncwarp();
            }
            kahan_add(sx, cx, tx); kahan_add(sy, cy, ty); kahan_add(sz, cz, tz);
            tx = ty = tz = 0.f;
        }
        nrg = 0;
        __syncwarp();
    };

    const int root = gal_root[wi.x];
    if (root < 1 || root >= n_cells) {
        bad = true;
    } else {
        if (lane == 0) stk[w][0] = root;
        nst = 1;
    }
    __syncwarp();
    while (nst > 0 && !bad) {
        if (++pops > max_pops) { bad = true; break; }
        const int c = stk[w][--nst];
        __syncwarp();
        const int4 pm = __ldg(&cell_meta[c]);
        const int F = pm.x, nch = (pm.w >> 4) & 15;
        if ((pm.w & 15) != BK_INTERNAL || F < 1 || nch > 8 || F + nch > n_cells) { bad = true; break; }
        bool a_cell = false, a_range = false, a_push = false, a_bad = false;
        float4 ccm = make_float4(0.f, 0.f, 0.f, 0.f);
        int first = 0, count = 0, ch = 0;
        if (lane < nch) {
            ch = F + lane;
            ccm = __ldg(&cell_com[ch]);
            const int4 mt = __ldg(&cell_meta[ch]);
            const int kind = mt.w & 15;
            count = __ldg(&cell_count[ch]);
            first = kind == BK_INTERNAL ? __ldg(&cell_first[ch]) : mt.x;
            const int level = (int)__ldg(&cell_hi[ch]).w;
            const float side = ldexpf(gb.w, kSlotLevels - level);
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
            // node data outside the body range would be a corrupt tree: report, never dereference
            if (a_range && (first < 0 || count < 0 || first + count > nbodies)) a_range = false, a_bad = true;
        }
        if (__any_sync(0xffffffffu, a_bad)) { bad = true; break; }
        const uint32_t bc = __ballot_sync(0xffffffffu, a_cell);
        if (bc) {
            if (ncl + __popc(bc) > kGCells) flush_cells();
            if (a_cell) {
                const int idx = ncl + __popc(bc & lt);
                lcm[w][idx] = ccm;
                lq1[w][idx] = __ldg(&cell_q1[ch]);
                lq2[w][idx] = __ldg(&cell_q2[ch]);
            }
            ncl += __popc(bc);
        }
        const uint32_t br = __ballot_sync(0xffffffffu, a_range);
        if (br) {
            if (nrg + __popc(br) > kGRanges) flush_ranges();
            if (a_range) lrg[w][nrg + __popc(br & lt)] = make_int2(first, count);
            nrg += __popc(br);
        }
        const uint32_t bp = __ballot_sync(0xffffffffu, a_push);
        if (bp) {
            if (nst + __popc(bp) > kGStack) { bad = true; break; }
            if (a_push) stk[w][nst + __popc(bp & lt)] = ch;
            nst += __popc(bp);
        }
        __syncwarp();
    }
    if (!bad) {
        flush_cells();
        flush_ranges();
    }
    kahan_add(sx, cx, tx); kahan_add(sy, cy, ty); kahan_add(sz, cz, tz);
    if (bad && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
    if (valid) acc[sorder[s]] = make_float4(G * (sx - cx), G * (sy - cy), G * (sz - cz), 0.f);
    unsigned long long cc2 = cnt;
    for (int o = 16; o > 0; o >>= 1) cc2 += __shfl_down_sync(0xffffffffu, cc2, o);
    if (lane == 0 && cc2) atomicAdd(inter, cc2);
}

// ---- batched direct sum --------------------------------------------------------
// unit = (first target body, first source tile, source tiles, index of the
// target's sum partial); the compensation partial follows at +comp_offset of
// the unit's galaxy, kept in unit_comp.
template <int LAW, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK) k_batch_direct(const float4* __restrict__ pos, const int4* __restrict__ units,
                                                        const int32_t* __restrict__ unit_comp, int nunits,
                                                        int* __restrict__ next_unit, float S,
                                                        float4* __restrict__ part) {
    __shared__ float4 tile[kDirTile];
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
                    for (int k = 0; k < IPT; ++k) interact<LAW>(pj, xi[k], yi[k], zi[k], S, tx[k], ty[k], tz[k]);
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
