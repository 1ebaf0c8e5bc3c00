// nb_tree.cu -- Barnes-Hut octree build on the GPU: K2 keys, K3 radix sort,
// K4 topology, K5 bottom-up mass and centre of mass.
//
// Replaces the serial pointer octree of BarnesHut::Update
// (src/Sim/BarnesHut.cpp:44-56) and Octree::Split/Add/CalculateMass
// (src/Sim/Octree.cpp:16-105) with the same tree, built in parallel:
//
//  * K2: a body's key is the octant path Octree::Add takes from the root,
//    3 bits per level, octant = x + 2y + 4z (src/Sim/Octree.cpp:25-41).  The
//    child bounds are replayed in float exactly as Split computes them
//    (cur += size, BottomRight = cur + size, Size = BottomRight.x - TopLeft.x),
//    with the half-open containment of BoundingCube::Contains
//    (src/Sim/Octree.hpp:18-22).  A body outside the root cube gets key ~0:
//    the reference drops it from the tree but counts it in the root.
//  * K3: stable LSD radix sort of (key, body) pairs, 8 passes of 8 bits, one
//    launch per pass: the digit histograms of all passes come with the keys,
//    and each pass ranks, finds its tile's offsets by decoupled look-back and
//    scatters in one kernel (the scatter ranks digits with warp match_any).
//    Passes whose digit is the same for every key are skipped on the device.
//  * K4: the reference tree splits a node when a second body arrives and
//    creates all 8 children, so its internal nodes are exactly the key
//    prefixes shared by at least two bodies (and the root whenever it holds
//    two bodies, dropped ones included).  With sorted keys, delta(s) = the
//    number of leading octants bodies s and s+1 share; position s starts the
//    internal nodes of levels delta(s-1)+1 .. min(delta(s), D-1) and one
//    leaf.  Internal nodes are numbered by (first body, level) through a
//    prefix sum; a node whose parent starts at an earlier body finds it in a
//    hash table keyed by (1 << 3 level) | prefix.  Each internal node stores
//    only its non-empty children, as consecutive cells in octant order
//    (empty children hold no mass and contribute exactly zero force).
//  * Depth cap D (max_depth, 21 = 63-bit keys): bodies sharing all D octants
//    form one leaf (a bucket).  A bucket's mass and centre of mass sum its
//    bodies in ascending body index (stable sort order).
//  * K5: CalculateMass in the same arithmetic: TotalMass is a double sum of
//    the children in octant order, CentreOfMass += child COM * float(child
//    mass) in float, then scaled by 1.f / float(TotalMass).  Nodes are
//    finished bottom-up: the last child to arrive finishes its parent.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include "nb_scan.cuh"
#include "nb_lookback.cuh"
#include "nb_morton.cuh"
#include "nb_cellrec.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace nb {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per tile
// a radix pass ranks a tile with more threads and fewer keys each (more warps
// in flight to hide the loads); at most 64 registers, two blocks per SM
constexpr int kPassThreads = 512;
constexpr int kPassWarps = kPassThreads / 32;
constexpr int kPassItems = kSortTile / kPassThreads;
constexpr int kPasses = 8;
constexpr int kEmitBlock = 256;

enum : int { KIND_SINGLE = 1, KIND_BUCKET = 2, KIND_INTERNAL = 3 };

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------- K2 keys --
// The octant path of body p (Octree::Add's descent) and its length; gap: the
// path met a gap between float child bounds and was cut short.
__device__ __forceinline__ uint64_t body_key(const float4 p, float half, int D, bool& inside, bool& gap, int& d) {
    float lo0 = -half, lo1 = -half, lo2 = -half, hi0 = half, hi1 = half, hi2 = half;
    inside = p.x >= lo0 && p.y >= lo1 && p.z >= lo2 && p.x < hi0 && p.y < hi1 && p.z < hi2;
    gap = false;
    d = 0;
    if (!inside) return ~0ull;
    uint64_t key = 0;
    float size = __fsub_rn(hi0, lo0);
    for (int l = 0; l < D; ++l) {
        const float s = __fmul_rn(size, 0.5f);   // Size / 2: exact halving, the same value as a division
        const float m0 = __fadd_rn(lo0, s), m1 = __fadd_rn(lo1, s), m2 = __fadd_rn(lo2, s);
        const float t0 = __fadd_rn(m0, s), t1 = __fadd_rn(m1, s), t2 = __fadd_rn(m2, s);
        int oct = 0;
        bool ok = true;
        if (p.x >= m0 && p.x < t0) { oct |= 1; lo0 = m0; hi0 = t0; }
        else if (p.x >= lo0 && p.x < m0) { hi0 = m0; }
        else ok = false;
        if (p.y >= m1 && p.y < t1) { oct |= 2; lo1 = m1; hi1 = t1; }
        else if (p.y >= lo1 && p.y < m1) { hi1 = m1; }
        else ok = false;
        if (p.z >= m2 && p.z < t2) { oct |= 4; lo2 = m2; hi2 = t2; }
        else if (p.z >= lo2 && p.z < m2) { hi2 = m2; }
        else ok = false;
        if (!ok) break;
        size = __fsub_rn(hi0, lo0);
        key = (key << 3) | (uint64_t)oct;
        ++d;
    }
    if (d < D) {   // a gap between float child bounds: left-align the path
        key <<= 3 * (D - d);
        gap = true;
    }
    return key;
}

// Zeroes this tile's look-back status words: every radix pass's, and the
// positions scan's.
__device__ __forceinline__ void zero_tile_status(unsigned long long* sort_status, int ntiles,
                                                 unsigned long long* pos_status) {
    for (int p = 0; p < kPasses; ++p)
        sort_status[((size_t)p * ntiles + blockIdx.x) * 256 + threadIdx.x] = 0ull;
    if (threadIdx.x == 0) pos_status[blockIdx.x] = 0ull;
}

// Radix passes that the top bits make redundant.  Keys are grouped by their
// top 4 bits (the root octant, and ~0 for bodies outside the root or tile
// padding), which the top pass sorts.  A lower pass whose digit is the same
// for every key of each group changes nothing in the final order: the top pass
// orders the groups, and within a group that digit is constant, so the order
// within the group is that of the passes below it.  Such a pass is skipped.
// For a galaxy at the centre of the reference's +-4000 cube, the bits of
// levels 2-7 are fixed within each root octant: two of the eight passes go.
// The group bits are recorded as two ORs per group, of the keys and of their
// complements (both start at zero with the counters): a bit varies within
// group g where both have it.
constexpr int kKeyGroups = 16;
__device__ __forceinline__ unsigned long long* group_bits(uint32_t* ghist) {
    return reinterpret_cast<unsigned long long*>(ghist + kPasses * 256);
}

// Adds a key to its group's bits in shared memory: one atomic pair per warp
// when the warp's keys share a group (the common case once keys are in
// galaxy or octant order), else one per lane.
__device__ __forceinline__ void note_group(uint64_t key, unsigned long long* sh) {
    const uint32_t g = (uint32_t)(key >> 60);
    const uint32_t g0 = __shfl_sync(0xffffffffu, g, 0);
    if (__all_sync(0xffffffffu, g == g0)) {
        const uint32_t lo = (uint32_t)key, hi = (uint32_t)(key >> 32);
        const unsigned long long o =
            ((unsigned long long)__reduce_or_sync(0xffffffffu, hi) << 32) | __reduce_or_sync(0xffffffffu, lo);
        const unsigned long long z =
            ((unsigned long long)__reduce_or_sync(0xffffffffu, ~hi) << 32) | __reduce_or_sync(0xffffffffu, ~lo);
        if ((threadIdx.x & 31) == 0) {
            atomicOr(&sh[g0], o);
            atomicOr(&sh[kKeyGroups + g0], z);
        }
    } else {
        atomicOr(&sh[g], (unsigned long long)key);
        atomicOr(&sh[kKeyGroups + g], (unsigned long long)~key);
    }
}

// Adds a tile's digit histograms of every pass into ghist (bins that are
// zero in this tile cost nothing), and its group bits after them.
__device__ __forceinline__ void flush_hist(uint32_t (*h)[256], const unsigned long long* sh_groups, uint32_t* ghist) {
    __syncthreads();
    for (int i = threadIdx.x; i < kPasses * 256; i += kSortThreads) {
        const uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(&ghist[i], v);
    }
    if (threadIdx.x < 2 * kKeyGroups && sh_groups[threadIdx.x])
        atomicOr(&group_bits(ghist)[threadIdx.x], sh_groups[threadIdx.x]);
}

// K2 + the radix sort's global histograms: one block per tile of kSortTile
// keys (key ~0 past n); counts bodies inside the root and paths cut by gaps.
__global__ void __launch_bounds__(kSortThreads) k_keys_hist(const float4* __restrict__ pos, int n, float half, int D,
                                                            uint64_t* __restrict__ keys, int32_t* __restrict__ vals,
                                                            int32_t* __restrict__ depth,
                                                            int32_t* __restrict__ counters, uint32_t* __restrict__ ghist,
                                                            unsigned long long* __restrict__ sort_status, int ntiles,
                                                            unsigned long long* __restrict__ pos_status) {
    __shared__ uint32_t h[kPasses][256];
    __shared__ unsigned long long sh_groups[2 * kKeyGroups];
    for (int i = threadIdx.x; i < kPasses * 256; i += kSortThreads) (&h[0][0])[i] = 0;
    if (threadIdx.x < 2 * kKeyGroups) sh_groups[threadIdx.x] = 0ull;
    zero_tile_status(sort_status, ntiles, pos_status);
    __syncthreads();
    for (int it = 0; it < kSortItems; ++it) {
        const int i = blockIdx.x * kSortTile + it * kSortThreads + threadIdx.x;
        vals[i] = i;
        bool inside = false, gap = false;
        uint64_t key = ~0ull;
        if (i < n) {
            int d;
            key = body_key(pos[i], half, D, inside, gap, d);
            depth[i] = d;
        }
        keys[i] = key;
#pragma unroll
        for (int p = 0; p < kPasses; ++p) atomicAdd(&h[p][(key >> (8 * p)) & 255], 1u);
        note_group(key, sh_groups);
        const uint32_t in_b = __ballot_sync(0xffffffffu, inside);
        const uint32_t gap_b = __ballot_sync(0xffffffffu, gap);
        if ((threadIdx.x & 31) == 0) {
            if (in_b) atomicAdd(&counters[TC_NIN], __popc(in_b));
            if (gap_b) atomicAdd(&counters[TC_GAPS], __popc(gap_b));
        }
    }
    flush_hist(h, sh_groups, ghist);
}

// ------------------------------------------------------------ K3 radix sort --
// plan[p] = 1 when pass p is skipped: every key has the same digit, or (below
// the top pass) every key of each top group has (note_group); plan[8+p] =
// buffer the pass reads; plan[16] = buffer holding the result.  dig_off[p][d] = keys
// with a smaller digit than d in pass p (where digit d's keys start).
__global__ void k_sort_plan(const uint32_t* __restrict__ ghist, int nk, int32_t* __restrict__ plan,
                            int32_t* __restrict__ dig_off) {
    __shared__ int triv[kPasses];
    __shared__ int sh_warp[33];
    // bits that vary within some top group
    __shared__ unsigned long long sh_var;
    if (threadIdx.x == 0) {
        const unsigned long long* gb = group_bits(const_cast<uint32_t*>(ghist));
        unsigned long long var = 0ull;
        for (int g = 0; g < kKeyGroups; ++g) var |= gb[g] & gb[kKeyGroups + g];
        sh_var = var;
    }
    __syncthreads();
    for (int p = 0; p < kPasses; ++p) {
        const int c = (int)ghist[p * 256 + threadIdx.x];
        const int t = __syncthreads_or(c == nk);
        if (threadIdx.x == 0) triv[p] = t || (p < kPasses - 1 && ((sh_var >> (8 * p)) & 255ull) == 0ull);
        int total;
        dig_off[p * 256 + threadIdx.x] = block_excl_scan(c, sh_warp, &total);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int cur = 0;
        for (int p = 0; p < kPasses; ++p) {
            plan[p] = triv[p];
            plan[8 + p] = cur;
            if (!triv[p]) cur ^= 1;
        }
        plan[16] = cur;
    }
}

// One pass of the stable LSD sort in one launch (the one-sweep scheme,
// Adinets and Merrill 2022): a tile ranks its keys by the pass's digit
// (warp match_any, warps in order: stable), publishes its digit counts and
// finds where earlier tiles put theirs by decoupled look-back, then scatters.
__global__ void __launch_bounds__(kPassThreads, 2) k_sort_pass(uint64_t* __restrict__ k0, uint64_t* __restrict__ k1,
                                                            int32_t* __restrict__ v0, int32_t* __restrict__ v1,
                                                            int ntiles, const int32_t* __restrict__ plan, int pass,
                                                            const int32_t* __restrict__ dig_off,
                                                            unsigned long long* __restrict__ status,
                                                            int* __restrict__ tile_ctr, int* __restrict__ err) {
    if (plan[pass]) return;
    const int src = plan[8 + pass];
    const uint64_t* ks = src ? k1 : k0;
    uint64_t* kd = src ? k0 : k1;
    const int32_t* vs = src ? v1 : v0;
    int32_t* vd = src ? v0 : v1;
    __shared__ uint32_t whist[kPassWarps][256];
    __shared__ int32_t gbase[256];
    __shared__ int sh_tile;
    const int tile = lb_tile_index(tile_ctr, &sh_tile);
    if (tile >= ntiles) return;   // cannot happen with one block per tile; kept as a guard
    for (int i = threadIdx.x; i < kPassWarps * 256; i += kPassThreads) (&whist[0][0])[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int shift = 8 * pass;
    const int base = tile * kSortTile + warp * (32 * kPassItems) + lane;
    uint64_t k[kPassItems];
    int32_t v[kPassItems];
    uint32_t r[kPassItems];
#pragma unroll
    for (int it = 0; it < kPassItems; ++it) {
        k[it] = ks[base + it * 32];
        v[it] = vs[base + it * 32];
    }
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int it = 0; it < kPassItems; ++it) {
        const uint32_t d = (uint32_t)(k[it] >> shift) & 255u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t b = whist[warp][d];
        r[it] = b + __popc(peers & lt);
        __syncwarp();
        if (lane == 31 - __clz(peers)) whist[warp][d] = b + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x < 256) {   // one thread per digit
        const int d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kPassWarps; ++w) {
            const uint32_t c = whist[w][d];
            whist[w][d] = run;
            run += c;
        }
        unsigned long long* st = status + (size_t)tile * 256 + d;
        uint32_t excl = 0;
        if (tile == 0) {
            lb_publish(st, 2u, run);
        } else {
            lb_publish(st, 1u, run);
            excl = lb_exclusive(status + d, tile, 256, err);
            lb_publish(st, 2u, excl + run);
        }
        gbase[d] = dig_off[pass * 256 + d] + (int)excl;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kPassItems; ++it) {
        const uint32_t d = (uint32_t)(k[it] >> shift) & 255u;
        const int dst = gbase[d] + (int)whist[warp][d] + (int)r[it];
        kd[dst] = k[it];
        vd[dst] = v[it];
    }
}

// --------------------------------------------------------- K4 topology ----
__device__ __forceinline__ int lcp_levels(uint64_t a, uint64_t b, int D) {
    const uint64_t x = a ^ b;
    if (x == 0) return D;
    return (__clzll((long long)x) - (64 - 3 * D)) / 3;
}

struct TopoView {
    const uint64_t* keys;     // sorted
    const int32_t* vals;      // body index per sorted position
    const int32_t* depth;     // per body (input order)
    int n_in, n_total, D;
    int int_cap, cell_cap;    // capacities of the internal-node and cell arrays
    __device__ int delta(int s) const {   // common levels of sorted bodies s and s+1; -1 past the end
        if (s < 0 || s + 1 >= n_in) return -1;
        int l = lcp_levels(keys[s], keys[s + 1], D);
        l = min(l, depth[vals[s]]);
        l = min(l, depth[vals[s + 1]]);
        return l;
    }
    // Nodes starting at sorted position s: internal levels lo..hi and a leaf at
    // level lf (lf = -1: s lies inside an earlier bucket).
    __device__ void info(int s, int& lo, int& hi, int& nint, int& lf, int& cur) const {
        const int prev = (s > 0) ? delta(s - 1) : -1;
        cur = delta(s);
        if (prev >= D) { lo = 0; hi = -1; nint = 0; lf = -1; return; }
        lo = prev + 1;
        hi = min(cur, D - 1);
        if (s == 0 && n_total >= 2) hi = max(hi, 0);
        nint = max(0, hi - lo + 1);
        lf = nint > 0 ? hi + 1 : lo;
    }
};

__device__ __forceinline__ uint64_t node_code(uint64_t key, int level, int D) {
    return (1ull << (3 * level)) | (level ? (key >> (3 * (D - level))) : 0ull);
}

__device__ __forceinline__ uint32_t hash_slot(uint64_t code, uint32_t mask) {
    uint64_t x = code * 0x9E3779B97F4A7C15ull;
    x ^= x >> 29;
    return (uint32_t)x & mask;
}

__device__ void hash_insert(uint64_t* hk, int32_t* hv, uint32_t mask, uint64_t code, int32_t val, int32_t* counters) {
    uint32_t h = hash_slot(code, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS((unsigned long long*)&hk[h], 0ull, (unsigned long long)code);
        if (prev == 0ull || prev == code) {
            hv[h] = val;
            return;
        }
        h = (h + 1) & mask;
    }
    atomicAdd(&counters[TC_HASHFAIL], 1);
}

__device__ int32_t hash_find(const uint64_t* hk, const int32_t* hv, uint32_t mask, uint64_t code, int32_t* counters) {
    uint32_t h = hash_slot(code, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint64_t k = hk[h];
        if (k == code) return hv[h];
        if (k == 0ull) break;
        h = (h + 1) & mask;
    }
    atomicAdd(&counters[TC_HASHFAIL], 1);
    return 0;
}

// Bounds of the node with the given code, replaying Octree::Split in float.
__device__ void node_bounds(uint64_t code, int level, float half, float3& lo, float3& hi, float& side) {
    lo = make_float3(-half, -half, -half);
    hi = make_float3(half, half, half);
    float size = __fsub_rn(hi.x, lo.x);
    for (int l = 1; l <= level; ++l) {
        const int dg = (int)((code >> (3 * (level - l))) & 7ull);
        const float s = __fmul_rn(size, 0.5f);   // Size / 2: exact halving, the same value as a division
        const float mx = __fadd_rn(lo.x, s), my = __fadd_rn(lo.y, s), mz = __fadd_rn(lo.z, s);
        if (dg & 1) { lo.x = mx; hi.x = __fadd_rn(mx, s); } else { hi.x = mx; }
        if (dg & 2) { lo.y = my; hi.y = __fadd_rn(my, s); } else { hi.y = my; }
        if (dg & 4) { lo.z = mz; hi.z = __fadd_rn(mz, s); } else { hi.z = mz; }
        size = __fsub_rn(hi.x, lo.x);
    }
    side = size;
}

// Positions in sorted order; brings the sort result to buffer 0 when the
// device plan left it in buffer 1 (no host read of the plan).
__global__ void k_gather_final(const float4* __restrict__ pos, uint64_t* __restrict__ k0,
                               const uint64_t* __restrict__ k1, int32_t* __restrict__ v0,
                               const int32_t* __restrict__ v1, int n, const int32_t* __restrict__ plan,
                               float4* __restrict__ spos) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const bool from1 = plan[16] != 0;
    const int v = from1 ? v1[s] : v0[s];
    if (from1) {
        k0[s] = k1[s];
        v0[s] = v;
    }
    spos[s] = (v >= 0 && v < n) ? pos[v] : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Internal nodes and leaf starting at sorted position s; bucket size and
// whether a bucket's bodies differ.
__device__ __forceinline__ void position_nodes(const TopoView& tv, const float4* spos, int s, int& nint, int& lf,
                                               int& count, bool& deeper) {
    int lo, hi, cur;
    count = 0;
    deeper = false;
    if (s < tv.n_in) {
        tv.info(s, lo, hi, nint, lf, cur);
    } else {
        nint = 0; lf = -1; cur = -1;
    }
    if (lf >= 0) {
        count = 1;
        if (lf == tv.D && cur == tv.D) {
            int x = s;
            const float4 p0 = spos[s];
            while (x + 1 < tv.n_in && tv.delta(x) == tv.D) {
                ++x;
                ++count;
                const float4 q = spos[x];
                if (q.x != p0.x || q.y != p0.y || q.z != p0.z) deeper = true;
            }
        }
    }
}

// Per tile of kSortTile sorted positions (kSortItems consecutive ones per
// thread): the nodes starting there, and the exclusive prefix of their
// internal-node counts by single-pass scan (pos_nint; the total goes to
// counters[TC_NINT]).  With hk_zero, the threads also clear the internal-node
// hash table for the emission that follows.
__global__ void __launch_bounds__(kSortThreads) k_positions_scan(TopoView tv, const float4* __restrict__ spos,
                                                                 int32_t* __restrict__ pos_nint,
                                                                 int32_t* __restrict__ leaf_level,
                                                                 int32_t* __restrict__ leaf_count,
                                                                 int32_t* __restrict__ counters,
                                                                 unsigned long long* __restrict__ status, int ntiles,
                                                                 uint64_t* __restrict__ hk_zero, int hk_n,
                                                                 int* __restrict__ err) {
    __shared__ int sh_warp[33], sh_off, sh_tile;
    if (hk_zero)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < hk_n; i += gridDim.x * blockDim.x) hk_zero[i] = 0ull;
    const int tile = lb_tile_index(&counters[TC_TILE_POS], &sh_tile);
    tv.n_in = counters[TC_NIN];
    const int s0 = tile * kSortTile + threadIdx.x * kSortItems;
    int nint[kSortItems];
    int sum = 0;
    unsigned nleaf = 0, ndeeper = 0;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int s = s0 + k;
        nint[k] = 0;
        if (s < tv.n_total) {
            int lf, count;
            bool deeper;
            position_nodes(tv, spos, s, nint[k], lf, count, deeper);
            leaf_level[s] = lf;
            leaf_count[s] = count;
            nleaf += lf >= 0 ? 1u : 0u;
            ndeeper += deeper ? 1u : 0u;
        }
        sum += nint[k];
    }
    for (int o = 16; o > 0; o >>= 1) {
        nleaf += __shfl_xor_sync(0xffffffffu, nleaf, o);
        ndeeper += __shfl_xor_sync(0xffffffffu, ndeeper, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (nleaf) atomicAdd(&counters[TC_NLEAF], (int)nleaf);
        if (ndeeper) atomicAdd(&counters[TC_DEEPER], (int)ndeeper);
    }
    int run = lb_scan_tile(sum, tile, ntiles, status, counters + TC_NINT, sh_warp, &sh_off, err);
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int s = s0 + k;
        if (s < tv.n_total) pos_nint[s] = run;
        run += nint[k];
    }
}

// Emits the internal nodes starting at each sorted position (level, first
// body, code, hash entry) and clears their child mask and counters, and the
// look-back status of the child-count scan.
__global__ void k_emit(TopoView tv, const int32_t* __restrict__ int_base, int32_t* __restrict__ int_level,
                       int32_t* __restrict__ int_first, uint64_t* __restrict__ int_code, uint64_t* __restrict__ hk,
                       int32_t* __restrict__ hv, uint32_t hmask, uint32_t* __restrict__ int_mask,
                       int32_t* __restrict__ int_nint, int32_t* __restrict__ int_pending,
                       int32_t* __restrict__ counters, unsigned long long* __restrict__ popc_status,
                       int popc_tiles) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = s; i < popc_tiles; i += gridDim.x * blockDim.x) popc_status[i] = 0ull;   // for k_popc_scan
    if (s >= tv.n_in) return;
    int lo, hi, nint, lf, cur;
    tv.info(s, lo, hi, nint, lf, cur);
    const uint64_t key = tv.keys[s];
    const int base = int_base[s];
    for (int l = lo; l <= hi; ++l) {
        const int k = base + (l - lo);
        if (k >= tv.int_cap) {
            atomicAdd(&counters[TC_OVERFLOW], 1);
            break;
        }
        const uint64_t code = node_code(key, l, tv.D);
        int_level[k] = l;
        int_first[k] = s;
        int_code[k] = code;
        int_mask[k] = 0u;
        int_nint[k] = 0;
        int_pending[k] = 0;
        hash_insert(hk, hv, hmask, code, k, counters);
    }
}

__device__ __forceinline__ void link_internal(int k, const int32_t* __restrict__ int_level,
                                              const int32_t* __restrict__ int_first,
                                              const uint64_t* __restrict__ int_code, const TopoView& tv, int ni,
                                              const uint64_t* __restrict__ hk, const int32_t* __restrict__ hv,
                                              uint32_t hmask, int32_t* __restrict__ int_parent,
                                              uint32_t* __restrict__ int_mask, int32_t* __restrict__ int_nint,
                                              int32_t* __restrict__ counters) {
    if (k >= ni || k == 0) return;
    const int l = int_level[k];
    const int s = int_first[k];
    const uint64_t code = int_code[k];
    const int prev = (s > 0) ? tv.delta(s - 1) : -1;
    const int parent = (l > prev + 1) ? k - 1 : hash_find(hk, hv, hmask, code >> 3, counters);
    if (parent < 0 || parent >= ni) {
        atomicAdd(&counters[TC_OVERFLOW], 1);
        return;
    }
    int_parent[k] = parent;
    atomicOr(&int_mask[parent], 1u << (unsigned)(code & 7ull));
    atomicAdd(&int_nint[parent], 1);
}

__device__ __forceinline__ void link_leaf(int s, const TopoView& tv, const int32_t* __restrict__ int_base,
                                          const int32_t* __restrict__ leaf_level, const uint64_t* __restrict__ hk,
                                          const int32_t* __restrict__ hv, uint32_t hmask,
                                          int32_t* __restrict__ leaf_parent, uint32_t* __restrict__ int_mask,
                                          int32_t* __restrict__ counters) {
    if (s >= tv.n_in) return;
    const int lf = leaf_level[s];
    if (lf <= 0) return;
    int lo, hi, nint, lf2, cur;
    tv.info(s, lo, hi, nint, lf2, cur);
    const uint64_t code = node_code(tv.keys[s], lf, tv.D);
    const int parent = nint > 0 ? int_base[s] + (lf - 1 - lo) : hash_find(hk, hv, hmask, code >> 3, counters);
    if (parent < 0 || parent >= tv.int_cap) {
        atomicAdd(&counters[TC_OVERFLOW], 1);
        return;
    }
    leaf_parent[s] = parent;
    atomicOr(&int_mask[parent], 1u << (unsigned)(code & 7ull));
}

// Every node's parent and the parents' child masks: blocks [0, int_blocks)
// link internal nodes, the rest link the leaf starting at each position.
// n_int_dev (graph builds) bounds the internal nodes by the device count.
__global__ void k_link(const int32_t* __restrict__ int_level, const int32_t* __restrict__ int_first,
                       const uint64_t* __restrict__ int_code, TopoView tv, int n_int,
                       const int32_t* __restrict__ n_int_dev, int int_blocks, const int32_t* __restrict__ int_base,
                       const int32_t* __restrict__ leaf_level, const uint64_t* __restrict__ hk,
                       const int32_t* __restrict__ hv, uint32_t hmask, int32_t* __restrict__ int_parent,
                       int32_t* __restrict__ leaf_parent, uint32_t* __restrict__ int_mask,
                       int32_t* __restrict__ int_nint, int32_t* __restrict__ counters) {
    if ((int)blockIdx.x < int_blocks) {
        const int k = blockIdx.x * blockDim.x + threadIdx.x;
        const int ni = n_int_dev ? min(*n_int_dev, n_int) : n_int;
        link_internal(k, int_level, int_first, int_code, tv, ni, hk, hv, hmask, int_parent, int_mask, int_nint,
                      counters);
    } else {
        const int s = (blockIdx.x - int_blocks) * blockDim.x + threadIdx.x;
        link_leaf(s, tv, int_base, leaf_level, hk, hv, hmask, leaf_parent, int_mask, counters);
    }
}

// int_block[k] = non-empty children of internal nodes before k (their first
// child cell, less one), by single-pass scan over tiles of kSortTile nodes.
__global__ void __launch_bounds__(kSortThreads) k_popc_scan(const uint32_t* __restrict__ mask, int n_int,
                                                            const int32_t* __restrict__ n_int_dev,
                                                            int32_t* __restrict__ out, int32_t* __restrict__ counters,
                                                            unsigned long long* __restrict__ status, int ntiles,
                                                            int* __restrict__ err) {
    __shared__ int sh_warp[33], sh_off, sh_tile;
    const int tile = lb_tile_index(&counters[TC_TILE_POPC], &sh_tile);
    const int ni = n_int_dev ? min(*n_int_dev, n_int) : n_int;
    const int k0 = tile * kSortTile + threadIdx.x * kSortItems;
    int c[kSortItems];
    int sum = 0;
    for (int k = 0; k < kSortItems; ++k) {
        c[k] = (k0 + k < ni) ? __popc(mask[k0 + k]) : 0;
        sum += c[k];
    }
    int run = lb_scan_tile(sum, tile, ntiles, status, nullptr, sh_warp, &sh_off, err);
    for (int k = 0; k < kSortItems; ++k) {
        if (k0 + k < n_int) out[k0 + k] = run;
        run += c[k];
    }
}

// Opening thresholds of a cell for the traversal: with r^2 computed exactly
// as the reference does, r^2 > accept_r2 guarantees float(side / r) < theta_f
// and r^2 < reject_r2 guarantees the opposite (1e-5 relative margins, far
// above the float rounding of the ratio); between the two the traversal
// evaluates the exactly rounded ratio.
__device__ __forceinline__ void open_thresholds(float side, float theta_f, int& accept_bits, int& reject_bits) {
    const double q = (double)side * (double)side / ((double)theta_f * (double)theta_f);
    accept_bits = __float_as_int(__double2float_ru(q * (1.0 + 1e-5)));
    reject_bits = __float_as_int(__double2float_rd(q * (1.0 - 1e-5)));
}

__device__ __forceinline__ int child_cell(const int32_t* int_block, const uint32_t* int_mask, int parent, int oct) {
    return 1 + int_block[parent] + __popc(int_mask[parent] & ((1u << oct) - 1u));
}

__device__ __forceinline__ void place_internal(int k, const int32_t* __restrict__ int_level,
                                               const uint64_t* __restrict__ int_code,
                                               const int32_t* __restrict__ int_parent,
                                               const uint32_t* __restrict__ int_mask,
                                               const int32_t* __restrict__ int_block, int ni, int cell_cap,
                                               float half, float theta_f, int32_t* __restrict__ int_cell,
                                               int4* __restrict__ cell_meta, float4* __restrict__ cell_lo,
                                               float4* __restrict__ cell_hi, uint64_t* __restrict__ cell_code,
                                               bool batch) {
    if (k >= ni) return;
    const uint64_t code = int_code[k];
    const int l = int_level[k];
    const int cell = (k == 0) ? 0 : child_cell(int_block, int_mask, int_parent[k], (int)(code & 7ull));
    if (cell >= cell_cap) {
        int_cell[k] = 0;
        return;
    }
    int_cell[k] = cell;
    if (batch) return;   // the batched form's moment pass writes the node's record
    float3 lo, hi;
    float side;
    node_bounds(code, l, half, lo, hi, side);
    const uint32_t m = int_mask[k];
    int ab, rb;
    open_thresholds(side, theta_f, ab, rb);
    cell_meta[cell] = make_int4(1 + int_block[k], ab, rb, KIND_INTERNAL | (__popc(m) << 4));
    cell_lo[cell] = make_float4(lo.x, lo.y, lo.z, side);
    cell_hi[cell] = make_float4(hi.x, hi.y, hi.z, (float)l);
    cell_code[cell] = code;
}

__device__ __forceinline__ void place_leaf(int s, const TopoView& tv, const int32_t* __restrict__ leaf_level,
                                           const int32_t* __restrict__ leaf_count,
                                           const int32_t* __restrict__ leaf_parent,
                                           const uint32_t* __restrict__ int_mask,
                                           const int32_t* __restrict__ int_block, const float4* __restrict__ spos,
                                           float half, float theta_f, float4* __restrict__ cell_com,
                                           double* __restrict__ cell_mass, int32_t* __restrict__ cell_count,
                                           int4* __restrict__ cell_meta, float4* __restrict__ cell_lo,
                                           float4* __restrict__ cell_hi, uint64_t* __restrict__ cell_code,
                                           CellRec* __restrict__ rec) {
    if (s >= tv.n_in) return;
    const int lf = leaf_level[s];
    if (lf < 0) return;
    const uint64_t code = node_code(tv.keys[s], lf, tv.D);
    if (lf > 0 && (leaf_parent[s] < 0 || leaf_parent[s] >= tv.int_cap)) return;   // parent lost to an overflow
    const int cell = (lf == 0) ? 0 : child_cell(int_block, int_mask, leaf_parent[s], (int)(code & 7ull));
    if (cell >= tv.cell_cap) return;
    if (rec) {   // the batched form: the leaf's whole record (bodies clamped to the sorted range)
        write_leaf_record(rec + cell, spos, s, max(1, min(leaf_count[s], tv.n_in - s)), lf);
        return;
    }
    float3 lo, hi;
    float side;
    node_bounds(code, lf, half, lo, hi, side);
    const int count = leaf_count[s];
    float4 com;
    double M;
    if (count == 1) {
        // leaf with one body: CentreOfMass = P->Position, TotalMass = P->Mass
        com = spos[s];
        M = (double)com.w;
    } else {
        // depth-cap bucket: bodies in ascending index order
        float cx = 0.f, cy = 0.f, cz = 0.f;
        M = 0.0;
        for (int q = s; q < s + count; ++q) {
            const float4 p = spos[q];
            M += (double)p.w;
            const float mf = p.w;
            cx = __fadd_rn(cx, __fmul_rn(p.x, mf));
            cy = __fadd_rn(cy, __fmul_rn(p.y, mf));
            cz = __fadd_rn(cz, __fmul_rn(p.z, mf));
        }
        if (M > 0.0) {
            const float inv = __fdiv_rn(1.0f, (float)M);
            cx = __fmul_rn(cx, inv); cy = __fmul_rn(cy, inv); cz = __fmul_rn(cz, inv);
        }
        com = make_float4(cx, cy, cz, (float)M);
    }
    com.w = (float)M;
    cell_com[cell] = com;
    cell_mass[cell] = M;
    int ab, rb;
    open_thresholds(side, theta_f, ab, rb);
    cell_meta[cell] = make_int4(s, ab, rb, (count == 1 ? KIND_SINGLE : KIND_BUCKET) | (count << 8));
    cell_count[cell] = count;
    cell_lo[cell] = make_float4(lo.x, lo.y, lo.z, side);
    cell_hi[cell] = make_float4(hi.x, hi.y, hi.z, (float)lf);
    cell_code[cell] = code;
}

// Every cell: blocks [0, int_blocks) place internal nodes (bounds, opening
// thresholds, first child), the rest the leaf starting at each position
// (bounds, thresholds, mass and centre of mass of its body or bucket).  With
// rec (the batched form) an internal node only gets its cell and a leaf its
// 64-byte record.
__global__ void k_place(const int32_t* __restrict__ int_level, const uint64_t* __restrict__ int_code,
                        const int32_t* __restrict__ int_parent, const uint32_t* __restrict__ int_mask,
                        const int32_t* __restrict__ int_block, int n_int, const int32_t* __restrict__ n_int_dev,
                        int int_blocks, TopoView tv, const int32_t* __restrict__ leaf_level,
                        const int32_t* __restrict__ leaf_count, const int32_t* __restrict__ leaf_parent,
                        const float4* __restrict__ spos, float half, float theta_f, int32_t* __restrict__ int_cell,
                        float4* __restrict__ cell_com, double* __restrict__ cell_mass,
                        int32_t* __restrict__ cell_count, int4* __restrict__ cell_meta, float4* __restrict__ cell_lo,
                        float4* __restrict__ cell_hi, uint64_t* __restrict__ cell_code, CellRec* __restrict__ rec) {
    if ((int)blockIdx.x < int_blocks) {
        const int k = blockIdx.x * blockDim.x + threadIdx.x;
        const int ni = n_int_dev ? min(*n_int_dev, n_int) : n_int;
        place_internal(k, int_level, int_code, int_parent, int_mask, int_block, ni, tv.cell_cap, half, theta_f,
                       int_cell, cell_meta, cell_lo, cell_hi, cell_code, rec != nullptr);
    } else {
        const int s = (blockIdx.x - int_blocks) * blockDim.x + threadIdx.x;
        place_leaf(s, tv, leaf_level, leaf_count, leaf_parent, int_mask, int_block, spos, half, theta_f, cell_com,
                   cell_mass, cell_count, cell_meta, cell_lo, cell_hi, cell_code, rec);
    }
}

// ------------------------------------------------------------- K5 mass ----
__device__ void finish_node(int k, const int32_t* int_cell, const int32_t* int_block, const uint32_t* int_mask,
                            float4* cell_com, double* cell_mass, int32_t* cell_count, int dropped) {
    const int c = int_cell[k];
    const int F = 1 + int_block[k];
    const int nch = __popc(int_mask[k]);
    double M = 0.0;
    float cx = 0.f, cy = 0.f, cz = 0.f;
    int count = 0;
    for (int j = 0; j < nch; ++j) {
        const double mc = __ldcg(&cell_mass[F + j]);
        const float4 cc = __ldcg(&cell_com[F + j]);
        const int cnt = __ldcg(&cell_count[F + j]);
        M += mc;
        const float mf = (float)mc;
        cx = __fadd_rn(cx, __fmul_rn(cc.x, mf));
        cy = __fadd_rn(cy, __fmul_rn(cc.y, mf));
        cz = __fadd_rn(cz, __fmul_rn(cc.z, mf));
        count += cnt;
    }
    if (M > 0.0) {
        const float inv = __fdiv_rn(1.0f, (float)M);
        cx = __fmul_rn(cx, inv); cy = __fmul_rn(cy, inv); cz = __fmul_rn(cz, inv);
    }
    if (k == 0) count += dropped;
    __stcg(&cell_com[c], make_float4(cx, cy, cz, (float)M));
    __stcg(&cell_mass[c], M);
    __stcg(&cell_count[c], count);
}

__global__ void k_mass(int n_int, const int32_t* __restrict__ n_int_dev, const int32_t* __restrict__ int_parent,
                       const int32_t* __restrict__ int_nint,
                       int32_t* __restrict__ int_pending, const int32_t* __restrict__ int_cell,
                       const int32_t* __restrict__ int_block, const uint32_t* __restrict__ int_mask,
                       float4* __restrict__ cell_com, double* __restrict__ cell_mass,
                       int32_t* __restrict__ cell_count, int dropped) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int ni = n_int_dev ? min(*n_int_dev, n_int) : n_int;
    if (k >= ni || int_nint[k] != 0) return;
    for (int guard = 0; guard < 64; ++guard) {   // a path has at most 22 internal nodes
        finish_node(k, int_cell, int_block, int_mask, cell_com, cell_mass, cell_count, dropped);
        if (k == 0) return;
        const int p = int_parent[k];
        const int old = atomic_add_acq_rel(&int_pending[p], 1);   // publishes this node, sees its siblings
        if (old != int_nint[p] - 1) return;
        k = p;
    }
}

// ------------------------------------------------- batched forest keys ----
// Keys of the batched form's Barnes-Hut bodies [0, n) (nb_morton.cuh), with
// the radix sort's histograms and the look-back status cleared, one block per
// sort tile; the first threads also write each galaxy's cube for the
// traversal.  Pad entries [n, tiles * kSortTile) get key ~0.
__global__ void __launch_bounds__(kSortThreads) k_batch_keys_hist(
    const float4* __restrict__ pos, const int32_t* __restrict__ body_slot, int n, const unsigned* __restrict__ box_bits,
    int nslot, float4* __restrict__ gal_box, uint64_t* __restrict__ keys, int32_t* __restrict__ vals,
    int32_t* __restrict__ depth, uint32_t* __restrict__ ghist, unsigned long long* __restrict__ sort_status,
    int ntiles, unsigned long long* __restrict__ pos_status) {
    __shared__ uint32_t h[kPasses][256];
    __shared__ unsigned long long sh_groups[2 * kKeyGroups];
    const int g = blockIdx.x * kSortThreads + threadIdx.x;
    if (g < nslot) gal_box[g] = gal_cube(box_bits, g);
    if ((int)blockIdx.x >= ntiles) return;   // blocks past the keys only write galaxy cubes (block-uniform)
    for (int i = threadIdx.x; i < kPasses * 256; i += kSortThreads) (&h[0][0])[i] = 0;
    if (threadIdx.x < 2 * kKeyGroups) sh_groups[threadIdx.x] = 0ull;
    zero_tile_status(sort_status, ntiles, pos_status);
    __syncthreads();
    for (int it = 0; it < kSortItems; ++it) {
        const int i = blockIdx.x * kSortTile + it * kSortThreads + threadIdx.x;
        vals[i] = i;
        uint64_t key = ~0ull;
        if (i < n) {
            const int slot = body_slot[i];
            key = forest_key(pos[i], slot, gal_cube(box_bits, slot));
            depth[i] = kBatchDepth;
        }
        keys[i] = key;
#pragma unroll
        for (int p = 0; p < kPasses; ++p) atomicAdd(&h[p][(key >> (8 * p)) & 255], 1u);
        note_group(key, sh_groups);
    }
    flush_hist(h, sh_groups, ghist);
}

// --------------------------------------------------------------- host ----
// Replaces *p by a buffer of `bytes` (the old one returned after the work
// queued on st).
static cudaError_t grow(void** p, size_t bytes, cudaStream_t st) {
    dev_free(*p, st);
    *p = nullptr;
    return dev_alloc(p, bytes);
}

#define NB_TRY(x)                               \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

static cudaError_t reserve_bodies(nb_sim* sim, size_t nk) {
    TreeBuffers& t = sim->tree;
    if (nk <= t.body_cap) return cudaSuccess;
    const size_t cap = nk;
    NB_TRY(grow((void**)&t.keys[0], cap * 8, sim->stream));
    NB_TRY(grow((void**)&t.keys[1], cap * 8, sim->stream));
    NB_TRY(grow((void**)&t.vals[0], cap * 4, sim->stream));
    NB_TRY(grow((void**)&t.vals[1], cap * 4, sim->stream));
    NB_TRY(grow((void**)&t.depth, cap * 4, sim->stream));
    NB_TRY(grow((void**)&t.spos, cap * 16, sim->stream));
    NB_TRY(grow((void**)&t.pos_nint, cap * 4, sim->stream));
    NB_TRY(grow((void**)&t.leaf_level, cap * 4, sim->stream));
    NB_TRY(grow((void**)&t.leaf_count, cap * 4, sim->stream));
    NB_TRY(grow((void**)&t.leaf_parent, cap * 4, sim->stream));
    const size_t ntiles = cap / kSortTile;
    NB_TRY(grow((void**)&t.sort_status, (size_t)kPasses * ntiles * 256 * sizeof(unsigned long long), sim->stream));
    NB_TRY(grow((void**)&t.pos_status, ntiles * sizeof(unsigned long long), sim->stream));
    if (!t.plan) NB_TRY(dev_alloc(&t.plan, 32 * 4));
    if (!t.dig_off) NB_TRY(dev_alloc(&t.dig_off, kPasses * 256 * 4));
    if (!t.counters) {
        // counters, tile counters of the look-back kernels, then the radix histograms
        NB_TRY(dev_alloc(&t.counters, (kCounterWords + kPasses * 256 + 4 * kKeyGroups) * 4));
        t.ghist = reinterpret_cast<uint32_t*>(t.counters + kCounterWords);
    }
    if (!t.h_counters) NB_TRY(cudaMallocHost(&t.h_counters, TC_COUNT * 4));
    if (!t.interactions) NB_TRY(dev_alloc(&t.interactions, sizeof(unsigned long long)));
    t.body_cap = cap;
    return cudaSuccess;
}

static cudaError_t reserve_nodes(nb_sim* sim, size_t n_int, size_t n_cells) {
    TreeBuffers& t = sim->tree;
    if (n_int > t.int_cap) {
        const size_t cap = n_int + n_int / 4 + 64;
        NB_TRY(grow((void**)&t.int_level, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_first, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_parent, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_mask, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_nint, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_pending, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_block, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_cell, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.int_code, cap * 8, sim->stream));
        // internal nodes can outnumber bodies (chains of one-child nodes above
        // close pairs): the child-count scan's status is sized by them
        NB_TRY(grow((void**)&t.popc_status, ((cap + kSortTile - 1) / kSortTile) * sizeof(unsigned long long), sim->stream));
        t.int_cap = cap;
        size_t h = 1024;
        while (h < 2 * cap) h <<= 1;
        NB_TRY(grow((void**)&t.hkeys, h * 8, sim->stream));
        NB_TRY(grow((void**)&t.hvals, h * 4, sim->stream));
        t.hash_cap = h;
    }
    if (n_cells > t.cell_cap) {
        const size_t cap = n_cells + n_cells / 4 + 64;
        NB_TRY(grow((void**)&t.cell_com, cap * 16, sim->stream));
        NB_TRY(grow((void**)&t.cell_meta, cap * 16, sim->stream));
        NB_TRY(grow((void**)&t.cell_mass, cap * 8, sim->stream));
        NB_TRY(grow((void**)&t.cell_count, cap * 4, sim->stream));
        NB_TRY(grow((void**)&t.cell_lo, cap * 16, sim->stream));
        NB_TRY(grow((void**)&t.cell_hi, cap * 16, sim->stream));
        NB_TRY(grow((void**)&t.cell_code, cap * 8, sim->stream));
        t.cell_cap = cap;
    }
    return cudaSuccess;
}

cudaError_t tree_reserve(nb_sim* sim) {
    return reserve_bodies(sim, pad_up(std::max<size_t>(sim->n, 1), kSortTile));
}

void tree_free(nb_sim* sim) {
    TreeBuffers& t = sim->tree;
    void* ptrs[] = {t.keys[0], t.keys[1], t.vals[0], t.vals[1], t.depth, t.spos, t.pos_nint, t.leaf_level,
                    t.leaf_count, t.leaf_parent, t.int_level, t.int_first, t.int_parent, t.int_mask, t.int_nint,
                    t.int_pending, t.int_block, t.int_cell, t.int_code, t.cell_com, t.cell_meta, t.cell_mass,
                    t.cell_lo, t.cell_hi, t.cell_code, t.cell_count, t.hkeys, t.hvals, t.sort_status, t.pos_status,
                    t.popc_status, t.dig_off, t.plan, t.counters, t.interactions};
    for (void* p : ptrs) dev_free(p, sim->stream);
    if (t.h_counters) cudaFreeHost(t.h_counters);
    t = TreeBuffers{};
}

float theta_float(double theta) {
    float f = (float)theta;
    if ((double)f < theta) f = std::nextafter(f, INFINITY);
    return f;
}

static TopoView topo_view(nb_sim* sim) {
    TreeBuffers& t = sim->tree;
    TopoView tv;
    tv.keys = t.keys[t.final_buf];
    tv.vals = t.vals[t.final_buf];
    tv.depth = t.depth;
    tv.n_in = t.n_in;
    tv.n_total = (int)sim->n;
    tv.D = sim->prm.max_depth;
    tv.int_cap = (int)t.int_cap;
    tv.cell_cap = (int)t.cell_cap;
    return tv;
}

// Clears the counters and histograms, then keys of the current positions into
// t.keys[0] (input order, t.vals[0] = identity) with their histograms.
static cudaError_t launch_keys(nb_sim* sim, size_t nk) {
    TreeBuffers& t = sim->tree;
    const int ntiles = (int)(nk / kSortTile);
    NB_TRY(cudaMemsetAsync(t.counters, 0, (kCounterWords + kPasses * 256 + 4 * kKeyGroups) * 4, sim->stream));
    PhaseScope ps(sim, NB_PHASE_KEYS);
    k_keys_hist<<<ntiles, kSortThreads, 0, sim->stream>>>(sim->pos, (int)sim->n, sim->prm.bounds_half,
                                                          sim->prm.max_depth, t.keys[0], t.vals[0], t.depth,
                                                          t.counters, t.ghist, t.sort_status, ntiles, t.pos_status);
    return cudaGetLastError();
}

// The radix sort of t.keys[0] / t.vals[0] (histograms already made): the
// device plan, then one launch per pass.
static cudaError_t launch_sort(nb_sim* sim, size_t nk) {
    TreeBuffers& t = sim->tree;
    const int ntiles = (int)(nk / kSortTile);
    cudaStream_t st = sim->stream;
    PhaseScope ps(sim, NB_PHASE_SORT, 1 + kPasses);
    k_sort_plan<<<1, 256, 0, st>>>(t.ghist, (int)nk, t.plan, t.dig_off);
    for (int p = 0; p < kPasses; ++p)
        k_sort_pass<<<ntiles, kPassThreads, 0, st>>>(t.keys[0], t.keys[1], t.vals[0], t.vals[1], ntiles, t.plan, p,
                                                     t.dig_off, t.sort_status + (size_t)p * ntiles * 256,
                                                     t.counters + TC_TILE_SORT + p, sim->d_err);
    return cudaGetLastError();
}

cudaError_t tree_build(nb_sim* sim) {
    TreeBuffers& t = sim->tree;
    const int n = (int)sim->n;
    const size_t nk = pad_up(std::max<size_t>(sim->n, 1), kSortTile);
    const int ntiles = (int)(nk / kSortTile);
    NB_TRY(tree_reserve(sim));
    cudaStream_t st = sim->stream;
    NB_TRY(launch_keys(sim, nk));
    NB_TRY(launch_sort(sim, nk));
    // The sort result's buffer is decided on the device (passes with a constant
    // digit are skipped): the gather brings it to buffer 0 when it ended in
    // buffer 1, so no host read is needed here.
    {
        PhaseScope ps(sim, NB_PHASE_TOPOLOGY, 2);
        k_gather_final<<<(n + 255) / 256, 256, 0, st>>>(sim->pos, t.keys[0], t.keys[1], t.vals[0], t.vals[1], n,
                                                        t.plan, t.spos);
        t.final_buf = 0;
        TopoView tv = topo_view(sim);
        k_positions_scan<<<ntiles, kSortThreads, 0, st>>>(tv, t.spos, t.pos_nint, t.leaf_level, t.leaf_count,
                                                          t.counters, t.pos_status, ntiles, nullptr, 0, sim->d_err);
        NB_TRY(cudaMemcpyAsync(t.h_counters, t.counters, TC_COUNT * 4, cudaMemcpyDeviceToHost, st));
        NB_TRY(cudaStreamSynchronize(st));
    }
    t.n_in = t.h_counters[TC_NIN];
    t.n_int = t.h_counters[TC_NINT];
    t.n_cells = t.n_int + t.h_counters[TC_NLEAF];
    t.trivial = (n < 2) || (t.n_in < 2 && t.n_int == 0) || t.n_in == 0;
    if (t.trivial) return cudaSuccess;
    NB_TRY(reserve_nodes(sim, (size_t)t.n_int, (size_t)t.n_cells));
    TopoView tv = topo_view(sim);
    const int ni = t.n_int;
    const float tf = theta_float(sim->prm.theta);
    const uint32_t hmask = (uint32_t)(t.hash_cap - 1);
    {
        PhaseScope ps(sim, NB_PHASE_TOPOLOGY, 4);
        NB_TRY(cudaMemsetAsync(t.hkeys, 0, t.hash_cap * 8, st));
        const int nbk = (t.n_in + kEmitBlock - 1) / kEmitBlock;
        const int ib = (ni + kEmitBlock - 1) / kEmitBlock;
        const int ptiles = (ni + kSortTile - 1) / kSortTile;
        k_emit<<<nbk, kEmitBlock, 0, st>>>(tv, t.pos_nint, t.int_level, t.int_first, t.int_code, t.hkeys, t.hvals,
                                          hmask, t.int_mask, t.int_nint, t.int_pending, t.counters, t.popc_status,
                                          ptiles);
        k_link<<<ib + nbk, kEmitBlock, 0, st>>>(t.int_level, t.int_first, t.int_code, tv, ni, nullptr, ib, t.pos_nint,
                                               t.leaf_level, t.hkeys, t.hvals, hmask, t.int_parent, t.leaf_parent,
                                               t.int_mask, t.int_nint, t.counters);
        k_popc_scan<<<ptiles, kSortThreads, 0, st>>>(t.int_mask, ni, nullptr, t.int_block, t.counters,
                                                     t.popc_status, ptiles, sim->d_err);
        k_place<<<ib + nbk, kEmitBlock, 0, st>>>(t.int_level, t.int_code, t.int_parent, t.int_mask, t.int_block, ni,
                                                nullptr, ib, tv, t.leaf_level, t.leaf_count, t.leaf_parent, t.spos,
                                                sim->prm.bounds_half, tf, t.int_cell, t.cell_com, t.cell_mass,
                                                t.cell_count, t.cell_meta, t.cell_lo, t.cell_hi, t.cell_code,
                                                nullptr);
        NB_TRY(cudaGetLastError());
    }
    {
        PhaseScope ps(sim, NB_PHASE_MASS);
        k_mass<<<(ni + 255) / 256, 256, 0, st>>>(ni, nullptr, t.int_parent, t.int_nint, t.int_pending, t.int_cell,
                                                t.int_block, t.int_mask, t.cell_com, t.cell_mass, t.cell_count,
                                                n - t.n_in);
        NB_TRY(cudaGetLastError());
    }
    sim->tree_valid = true;
    return cudaSuccess;
}

cudaError_t tree_sizes(nb_sim* sim, int32_t* cells, int32_t* internal) {
    if (cells) *cells = sim->tree.trivial ? 0 : sim->tree.n_cells;
    if (internal) *internal = sim->tree.trivial ? 0 : sim->tree.n_int;
    return cudaSuccess;
}

// Keys of the current positions in input order (for export).
cudaError_t tree_keys_export(nb_sim* sim, uint64_t* d_keys, int32_t* d_depth) {
    TreeBuffers& t = sim->tree;
    const size_t nk = pad_up(std::max<size_t>(sim->n, 1), kSortTile);
    NB_TRY(tree_reserve(sim));
    NB_TRY(launch_keys(sim, nk));
    NB_TRY(cudaMemcpyAsync(d_keys, t.keys[0], sim->n * 8, cudaMemcpyDeviceToDevice, sim->stream));
    NB_TRY(cudaMemcpyAsync(d_depth, t.depth, sim->n * 4, cudaMemcpyDeviceToDevice, sim->stream));
    sim->tree_valid = false;   // the sort buffers no longer match the tree
    return cudaSuccess;
}

}  // namespace nb

// ----------------------------------------------------------------------------
// Topology without host synchronisation, for the batched form (its steps are
// captured in a CUDA graph).  The batched step's first kernel clears the
// counters and histograms and sets TC_NIN = n; tree_batch_keys writes the
// keys of bodies [0, n), their histograms and clears the look-back status
// (every body lies inside its cube).  Grid sizes come from the capacities;
// the kernels read the node counts on the device and report overflow in
// counters[TC_OVERFLOW].
// ----------------------------------------------------------------------------
namespace nb {

int tree_counter_words() { return kCounterWords + kPasses * 256 + 4 * kKeyGroups; }

cudaError_t tree_batch_keys(nb_sim* sim, const float4* pos, const int32_t* body_slot, int n,
                            const unsigned* box_bits, int nslot, float4* gal_box) {
    TreeBuffers& t = sim->tree;
    const int ntiles = (int)(pad_up(std::max<size_t>((size_t)n, 1), kSortTile) / kSortTile);
    const int blocks = std::max(ntiles, (nslot + kSortThreads - 1) / kSortThreads);
    PhaseScope ps(sim, NB_PHASE_KEYS);
    k_batch_keys_hist<<<blocks, kSortThreads, 0, sim->stream>>>(pos, body_slot, n, box_bits, nslot, gal_box,
                                                                t.keys[0], t.vals[0], t.depth, t.ghist,
                                                                t.sort_status, ntiles, t.pos_status);
    return cudaGetLastError();
}

cudaError_t tree_build_graph(nb_sim* sim, const float4* pos, int n, int D, bool counts_only, CellRec* rec) {
    TreeBuffers& t = sim->tree;
    const size_t nk = pad_up(std::max<size_t>((size_t)n, 1), kSortTile);
    const int ntiles = (int)(nk / kSortTile);
    cudaStream_t st = sim->stream;
    NB_TRY(launch_sort(sim, nk));
    t.final_buf = 0;
    t.n_in = n;
    TopoView tv;
    tv.keys = t.keys[0];
    tv.vals = t.vals[0];
    tv.depth = t.depth;
    tv.n_in = n;
    tv.n_total = n;
    tv.D = D;
    tv.int_cap = (int)t.int_cap;
    tv.cell_cap = (int)t.cell_cap;
    const int icap = (int)t.int_cap;
    const uint32_t hmask = (uint32_t)(t.hash_cap - 1);
    const int nbk = (n + kEmitBlock - 1) / kEmitBlock;
    const int ib = (icap + kEmitBlock - 1) / kEmitBlock;
    const int ptiles = (icap + kSortTile - 1) / kSortTile;
    PhaseScope ps(sim, NB_PHASE_TOPOLOGY, 6);
    k_gather_final<<<(n + 255) / 256, 256, 0, st>>>(pos, t.keys[0], t.keys[1], t.vals[0], t.vals[1], n, t.plan,
                                                    t.spos);
    // this scan also clears the internal-node hash table for the emission
    k_positions_scan<<<ntiles, kSortThreads, 0, st>>>(tv, t.spos, t.pos_nint, t.leaf_level, t.leaf_count, t.counters,
                                                      t.pos_status, ntiles, counts_only ? nullptr : t.hkeys,
                                                      (int)t.hash_cap, sim->d_err);
    if (counts_only) return cudaGetLastError();   // the node counts are in counters[TC_NINT], [TC_NLEAF]
    k_emit<<<nbk, kEmitBlock, 0, st>>>(tv, t.pos_nint, t.int_level, t.int_first, t.int_code, t.hkeys, t.hvals, hmask,
                                      t.int_mask, t.int_nint, t.int_pending, t.counters, t.popc_status, ptiles);
    k_link<<<ib + nbk, kEmitBlock, 0, st>>>(t.int_level, t.int_first, t.int_code, tv, icap, t.counters + TC_NINT, ib,
                                           t.pos_nint, t.leaf_level, t.hkeys, t.hvals, hmask, t.int_parent,
                                           t.leaf_parent, t.int_mask, t.int_nint, t.counters);
    k_popc_scan<<<ptiles, kSortThreads, 0, st>>>(t.int_mask, icap, t.counters + TC_NINT, t.int_block, t.counters,
                                                 t.popc_status, ptiles, sim->d_err);
    k_place<<<ib + nbk, kEmitBlock, 0, st>>>(t.int_level, t.int_code, t.int_parent, t.int_mask, t.int_block, icap,
                                            t.counters + TC_NINT, ib, tv, t.leaf_level, t.leaf_count, t.leaf_parent,
                                            t.spos, sim->prm.bounds_half, 1.0f, t.int_cell, t.cell_com, t.cell_mass,
                                            t.cell_count, t.cell_meta, t.cell_lo, t.cell_hi, t.cell_code, rec);
    return cudaGetLastError();
}

// Capacity of the node arrays for a batched build: exact counts are measured
// once with a synchronising build and doubled (positions evolve).
cudaError_t tree_reserve_graph(nb_sim* sim, int n, size_t n_int, size_t n_cells) {
    const size_t nk = pad_up(std::max<size_t>((size_t)n, 1), kSortTile);
    NB_TRY(reserve_bodies(sim, nk));
    return reserve_nodes(sim, n_int, n_cells);
}

int tree_sort_tile() { return kSortTile; }

}  // namespace nb
