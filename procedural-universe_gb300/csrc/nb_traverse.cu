// nb_traverse.cu -- K6: warp-cooperative Barnes-Hut traversal, and the
// octree export of the C-ABI.
//
// Replaces Octree::CalculateForce (src/Sim/Octree.cpp:107-145) called for
// every body by BarnesHut::Exec (src/Sim/BarnesHut.cpp:103-110).
//
// A warp owns 64 consecutive bodies of the key-sorted order, two per lane
// (spatially close, so their walks mostly coincide).  The warp shares one
// node stack in shared memory; an entry is (child range of a cell, lane mask
// per body slot): the bodies that decided to open that cell.  Popping an
// entry, lanes 0..7 load the
// cell's non-empty children (one coalesced load) into a per-warp shared
// buffer, and each lane of the mask applies the reference's per-body rule to
// every child, so each body makes exactly the decisions of the CPU recursion:
//   * a one-body leaf (NumParticles == 1): pairwise force unless it is the
//     body itself (p != P; with the float bounds nesting exactly, the
//     reference's !Bounds.Contains(p) holds for every other body);
//   * any other node: r = |p - COM| in float, d = side; if d / r < Theta the
//     monopole (COM, TotalMass) acts, else an internal node is opened
//     (__ballot_sync collects the lanes that open it into the pushed entry)
//     and a depth-cap bucket acts body by body.
// The opening test compares the float r^2 (computed as the reference does)
// with the cell's precomputed accept / reject thresholds; only when r^2 falls
// between them (a 2e-5 relative band) is the exactly rounded ratio
// float(side / sqrtf(r^2)) compared with theta_f, the smallest float >= Theta.
// Forces are summed in FP32 per popped cell and folded into a Kahan total.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include <cmath>
#include <vector>

namespace nb {

constexpr int kTravBlock = 128;
constexpr int kTravWarps = kTravBlock / 32;
constexpr int kTravBodies = 64;   // bodies per warp: two per lane
constexpr int kStack = 384;   // stack entries per warp (a walk step pushes at most 32)
constexpr float kTravTiny = 1e-30f;
constexpr unsigned kRangeBits = 28;   // stack entry: first child cell (28 bits) | child count << 28

enum : int { TK_SINGLE = 1, TK_BUCKET = 2, TK_INTERNAL = 3 };

template <int LAW>
__device__ __forceinline__ void pair_accel(float dx, float dy, float dz, float r2, float m, float S, float& ax,
                                           float& ay, float& az) {
    float w;
    if (LAW == NB_LAW_REFERENCE) {
        const float s = r2 + S;
        w = m * rsqrt_approx(fmaf(r2 * s, s, kTravTiny));
    } else {
        const float inv = rsqrt_approx(r2 + S);
        w = m * inv * (inv * inv);
    }
    ax = fmaf(w, dx, ax);
    ay = fmaf(w, dy, ay);
    az = fmaf(w, dz, az);
}

}  // namespace nb

#include "nb_traverse_kernel.cuh"

namespace nb {

cudaError_t tree_forces(nb_sim* sim) {
    TreeBuffers& t = sim->tree;
    cudaStream_t st = sim->stream;
    cudaError_t e = cudaMemsetAsync(t.interactions, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (t.trivial) {
        sim->inter_last = 0;
        return cudaMemsetAsync(sim->acc, 0, sim->n_pad * sizeof(float4), st);
    }
    const int n = (int)sim->n;
    const float tf = theta_float(sim->prm.theta);
    const float S = (float)sim->prm.softening2;
    const float G = (float)sim->prm.G;
    PhaseScope ps(sim, NB_PHASE_TRAVERSE);
    const int blocks = (n + kTravWarps * kTravBodies - 1) / (kTravWarps * kTravBodies);
#define NB_TRAV(L)                                                                                          \
    k_traverse<L><<<blocks, kTravBlock, 0, st>>>(t.spos, t.vals[t.final_buf], n, t.cell_com, t.cell_meta,   \
                                                 t.cell_lo, t.n_cells, t.n_int + 1, tf, S, G, sim->acc,     \
                                                 t.interactions, sim->d_err)
    if (sim->prm.law == NB_LAW_PLUMMER) NB_TRAV(NB_LAW_PLUMMER);
    else NB_TRAV(NB_LAW_REFERENCE);
#undef NB_TRAV
    return cudaGetLastError();
}

cudaError_t tree_keys_export(nb_sim* sim, uint64_t* d_keys, int32_t* d_depth);

}  // namespace nb

// ---------------------------------------------------------------- C-ABI ----
using namespace nb;

namespace {

int tfail(nb_sim* s, int code, const std::string& msg) {
    s->err = msg;
    return code;
}

int ensure_tree(nb_sim* s) {
    if (s->n == 0) return tfail(s, NB_EBADSTATE, "no particles");
    if (!s->tree_valid) {
        cudaError_t e = tree_build(s);
        if (e != cudaSuccess) return tfail(s, NB_ECUDA, std::string("tree_build: ") + cudaGetErrorString(e));
    }
    return nb_synchronize(s);
}

}  // namespace

extern "C" {

int nb_tree_keys(nb_sim* s, uint64_t* keys, int32_t* depth) {
    try {
        if (!s || !keys || !depth) return NB_EINVAL;
        if (s->n == 0) return NB_OK;
        cudaSetDevice(s->dev);
        uint64_t* dk = nullptr;
        int32_t* dd = nullptr;
        cudaError_t e = cudaMallocAsync(&dk, s->n * 8, s->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&dd, s->n * 4, s->stream);
        if (e == cudaSuccess) e = tree_keys_export(s, dk, dd);
        if (e == cudaSuccess) e = cudaMemcpyAsync(keys, dk, s->n * 8, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(depth, dd, s->n * 4, cudaMemcpyDeviceToHost, s->stream);
        if (dk) cudaFreeAsync(dk, s->stream);
        if (dd) cudaFreeAsync(dd, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return tfail(s, NB_ECUDA, std::string("nb_tree_keys: ") + cudaGetErrorString(e));
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_tree_size(nb_sim* s, size_t* nodes) {
    try {
        if (!s || !nodes) return NB_EINVAL;
        cudaSetDevice(s->dev);
        int rc = ensure_tree(s);
        if (rc) return rc;
        *nodes = s->tree.trivial ? 0 : (size_t)s->tree.n_cells;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_tree_stats(nb_sim* s, int64_t* stats8) {
    try {
        if (!s || !stats8) return NB_EINVAL;
        cudaSetDevice(s->dev);
        int rc = ensure_tree(s);
        if (rc) return rc;
        int32_t h[TC_COUNT] = {0};
        cudaError_t e = cudaMemcpy(h, s->tree.counters, sizeof(h), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return tfail(s, NB_ECUDA, cudaGetErrorString(e));
        stats8[0] = h[TC_NIN];
        stats8[1] = s->tree.trivial ? 0 : h[TC_NINT];
        stats8[2] = s->tree.trivial ? 0 : s->tree.n_cells;
        stats8[3] = h[TC_GAPS];
        stats8[4] = h[TC_DEEPER];
        stats8[5] = h[TC_HASHFAIL];
        stats8[6] = (int64_t)s->n - h[TC_NIN];
        stats8[7] = h[TC_OVERFLOW];
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_tree_nodes(nb_sim* s, nb_tree_node* nodes, size_t capacity) {
    try {
        if (!s || (!nodes && capacity)) return NB_EINVAL;
        cudaSetDevice(s->dev);
        int rc = ensure_tree(s);
        if (rc) return rc;
        const TreeBuffers& t = s->tree;
        if (t.trivial) return NB_OK;
        const size_t C = (size_t)t.n_cells;
        if (capacity < C) return tfail(s, NB_EINVAL, "capacity below nb_tree_size");
        std::vector<float4> com(C), lo(C), hi(C);
        std::vector<int4> meta(C);
        std::vector<double> mass(C);
        std::vector<uint64_t> code(C);
        std::vector<int32_t> order(s->n), count(C);
        cudaError_t e = cudaMemcpy(com.data(), t.cell_com, C * 16, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(count.data(), t.cell_count, C * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(lo.data(), t.cell_lo, C * 16, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(hi.data(), t.cell_hi, C * 16, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(meta.data(), t.cell_meta, C * 16, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(mass.data(), t.cell_mass, C * 8, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(code.data(), t.cell_code, C * 8, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(order.data(), t.vals[t.final_buf], s->n * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return tfail(s, NB_ECUDA, std::string("nb_tree_nodes: ") + cudaGetErrorString(e));
        for (size_t c = 0; c < C; ++c) {
            nb_tree_node& o = nodes[c];
            const int level = (int)hi[c].w;
            const int kind = meta[c].w & 15;
            o.level = level;
            o.count = count[c];
            o.first_child = kind == TK_INTERNAL ? meta[c].x : -1;
            o.body = kind == TK_SINGLE ? order[meta[c].x] : -1;
            o.prefix = level ? (code[c] & ((1ull << (3 * level)) - 1ull)) : 0ull;
            o.mass = mass[c];
            o.com[0] = com[c].x; o.com[1] = com[c].y; o.com[2] = com[c].z;
            o.side = lo[c].w;
            o.lo[0] = lo[c].x; o.lo[1] = lo[c].y; o.lo[2] = lo[c].z;
            o.bucket_begin = kind == TK_BUCKET ? meta[c].x : -1;
            o.bucket_end = kind == TK_BUCKET ? meta[c].x + count[c] : -1;
        }
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_tree_order(nb_sim* s, int32_t* order) {
    try {
        if (!s || !order) return NB_EINVAL;
        cudaSetDevice(s->dev);
        int rc = ensure_tree(s);
        if (rc) return rc;
        cudaError_t e = cudaMemcpy(order, s->tree.vals[s->tree.final_buf], s->n * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return tfail(s, NB_ECUDA, cudaGetErrorString(e));
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

}  // extern "C"
