// nb_traverse.cu -- K6: warp-cooperative Barnes-Hut traversal, and the
// octree export of the C-ABI.
//
// Replaces Octree::CalculateForce (src/Sim/Octree.cpp:107-145) called for
// every body by BarnesHut::Exec (src/Sim/BarnesHut.cpp:103-110).
//
// A warp owns 32 consecutive bodies of the key-sorted order (spatially
// close, so their walks mostly coincide).  The warp shares one node stack in
// shared memory; an entry is (cell, lane mask): the lanes that decided to
// open that cell.  Popping a cell, the warp visits its children; each lane in
// the mask applies the reference's per-body rule to each child, so every
// body makes exactly the decisions of the CPU recursion:
//   * a one-body leaf (NumParticles == 1): pairwise force unless it is the
//     body itself (p != P; with the float bounds nesting exactly, the
//     reference's !Bounds.Contains(p) holds for every other body);
//   * any other node: r = |p - COM| in float, d = side; if d / r < Theta the
//     monopole (COM, TotalMass) acts, else an internal node is opened
//     (__ballot_sync collects the lanes that open it into the pushed entry)
//     and a depth-cap bucket acts body by body.
// The comparison is the reference's float ratio against the double Theta,
// i.e. d / r < theta_f with theta_f the smallest float >= Theta.  It is
// decided from d^2 against theta_f^2 r^2 when that is clear by a 1e-5 margin,
// else by the exactly rounded sqrt and division, so decisions are exact.
// Forces are summed in FP32 per popped cell and folded into a Kahan total.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include <cmath>
#include <vector>

namespace nb {

constexpr int kTravBlock = 128;
constexpr int kTravWarps = kTravBlock / 32;
constexpr int kStack = 176;   // >= 7 * 21 + 8 entries: the deepest possible walk
constexpr float kTravTiny = 1e-30f;

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

template <int LAW>
__global__ void __launch_bounds__(kTravBlock) k_traverse(const float4* __restrict__ spos,
                                                         const int32_t* __restrict__ sorder, int n,
                                                         const float4* __restrict__ cell_com,
                                                         const int4* __restrict__ cell_meta, int n_cells,
                                                         int max_pops, float theta_f,
                                                         float th2, float S, float G, float4* __restrict__ acc,
                                                         unsigned long long* __restrict__ inter,
                                                         int* __restrict__ err) {
    __shared__ int2 stk[kTravWarps][kStack];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = (blockIdx.x * kTravWarps + w) * 32 + lane;
    const bool valid = s < n;
    const float4 p = valid ? spos[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    unsigned cnt = 0;

    auto visit = [&](int c, bool mine) -> bool {
        const float4 cm = __ldg(&cell_com[c]);
        const int4 mt = __ldg(&cell_meta[c]);
        const int kind = mt.w & 15;
        bool open = false;
        if (mine) {
            if (kind == TK_SINGLE) {
                if (mt.x != s) {
                    const float dx = cm.x - p.x, dy = cm.y - p.y, dz = cm.z - p.z;
                    pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), cm.w, S, tx, ty, tz);
                    ++cnt;
                }
            } else {
                const float dvx = __fsub_rn(p.x, cm.x), dvy = __fsub_rn(p.y, cm.y), dvz = __fsub_rn(p.z, cm.z);
                const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dvx, dvx), __fmul_rn(dvy, dvy)), __fmul_rn(dvz, dvz));
                const float side = __int_as_float(mt.z);
                const float d2 = __fmul_rn(side, side);
                const float t = __fmul_rn(th2, r2);
                bool accept;
                if (d2 < __fmul_rn(t, 0.99999f)) accept = true;
                else if (d2 > __fmul_rn(t, 1.00001f)) accept = false;
                else accept = __fdiv_rn(side, __fsqrt_rn(r2)) < theta_f;
                if (accept) {
                    if (cm.w != 0.f) {
                        pair_accel<LAW>(-dvx, -dvy, -dvz, r2, cm.w, S, tx, ty, tz);
                        ++cnt;
                    }
                } else if (kind == TK_INTERNAL) {
                    open = true;
                } else {
                    const int qe = min(mt.x + mt.y, n);
                    for (int q = max(mt.x, 0); q < qe; ++q) {
                        if (q == s) continue;
                        const float4 b = spos[q];
                        const float dx = b.x - p.x, dy = b.y - p.y, dz = b.z - p.z;
                        pair_accel<LAW>(dx, dy, dz, fmaf(dz, dz, fmaf(dy, dy, dx * dx)), b.w, S, tx, ty, tz);
                        ++cnt;
                    }
                }
            }
        }
        return open;
    };

    int top = 0;
    bool overflow = false;
    int pops = 0;
    {
        const unsigned om = __ballot_sync(0xffffffffu, visit(0, valid));
        if (om) {
            if (lane == 0) stk[w][0] = make_int2(0, (int)om);
            top = 1;
        }
    }
    __syncwarp();
    while (top > 0) {
        --top;
        const int2 e = stk[w][top];
        __syncwarp();
        const bool mine = ((unsigned)e.y >> lane) & 1u;
        const int4 pm = __ldg(&cell_meta[e.x]);
        const int F = pm.x, nch = pm.w >> 4;
        // A well-formed tree pops each internal cell at most once per warp and
        // keeps child ranges inside the cell array; anything else is reported.
        if (++pops > max_pops || F < 1 || nch > 8 || F + nch > n_cells) {
            overflow = true;
            break;
        }
        for (int j = 0; j < nch; ++j) {
            const unsigned b = __ballot_sync(0xffffffffu, visit(F + j, mine));
            if (b) {
                if (top < kStack) {
                    if (lane == 0) stk[w][top] = make_int2(F + j, (int)b);
                    ++top;
                } else {
                    overflow = true;
                }
            }
        }
        __syncwarp();
        kahan_add(sx, cx, tx);
        kahan_add(sy, cy, ty);
        kahan_add(sz, cz, tz);
        tx = ty = tz = 0.f;
        if (overflow) break;
    }
    kahan_add(sx, cx, tx);
    kahan_add(sy, cy, ty);
    kahan_add(sz, cz, tz);
    if (overflow && lane == 0) record_error(err, DEV_STACK_OVERFLOW);
    if (valid) acc[sorder[s]] = make_float4(G * (sx - cx), G * (sy - cy), G * (sz - cz), 0.f);
    unsigned long long c = cnt;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(inter, c);
}

static float theta_float(double theta) {
    float f = (float)theta;
    if ((double)f < theta) f = std::nextafter(f, INFINITY);
    return f;
}

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
    const float th2 = tf * tf;
    const float S = (float)sim->prm.softening2;
    const float G = (float)sim->prm.G;
    const int blocks = (n + kTravBlock - 1) / kTravBlock;
    PhaseScope ps(sim, NB_PHASE_TRAVERSE);
    if (sim->prm.law == NB_LAW_PLUMMER)
        k_traverse<NB_LAW_PLUMMER><<<blocks, kTravBlock, 0, st>>>(t.spos, t.vals[t.final_buf], n, t.cell_com,
                                                                 t.cell_meta, t.n_cells, t.n_int + 1, tf, th2, S, G,
                                                                 sim->acc,
                                                                 t.interactions, sim->d_err);
    else
        k_traverse<NB_LAW_REFERENCE><<<blocks, kTravBlock, 0, st>>>(t.spos, t.vals[t.final_buf], n, t.cell_com,
                                                                   t.cell_meta, t.n_cells, t.n_int + 1, tf, th2, S,
                                                                   G, sim->acc,
                                                                   t.interactions, sim->d_err);
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
}

int nb_tree_size(nb_sim* s, size_t* nodes) {
    if (!s || !nodes) return NB_EINVAL;
    cudaSetDevice(s->dev);
    int rc = ensure_tree(s);
    if (rc) return rc;
    *nodes = s->tree.trivial ? 0 : (size_t)s->tree.n_cells;
    return NB_OK;
}

int nb_tree_stats(nb_sim* s, int64_t* stats8) {
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
    stats8[7] = 0;
    return NB_OK;
}

int nb_tree_nodes(nb_sim* s, nb_tree_node* nodes, size_t capacity) {
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
    std::vector<int32_t> order(s->n);
    cudaError_t e = cudaMemcpy(com.data(), t.cell_com, C * 16, cudaMemcpyDeviceToHost);
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
        o.count = meta[c].y;
        o.first_child = kind == TK_INTERNAL ? meta[c].x : -1;
        o.body = kind == TK_SINGLE ? order[meta[c].x] : -1;
        o.prefix = level ? (code[c] & ((1ull << (3 * level)) - 1ull)) : 0ull;
        o.mass = mass[c];
        o.com[0] = com[c].x; o.com[1] = com[c].y; o.com[2] = com[c].z;
        o.side = lo[c].w;
        o.lo[0] = lo[c].x; o.lo[1] = lo[c].y; o.lo[2] = lo[c].z;
        o.bucket_begin = kind == TK_BUCKET ? meta[c].x : -1;
        o.bucket_end = kind == TK_BUCKET ? meta[c].x + meta[c].y : -1;
    }
    return NB_OK;
}

int nb_tree_order(nb_sim* s, int32_t* order) {
    if (!s || !order) return NB_EINVAL;
    cudaSetDevice(s->dev);
    int rc = ensure_tree(s);
    if (rc) return rc;
    cudaError_t e = cudaMemcpy(order, s->tree.vals[s->tree.final_buf], s->n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return tfail(s, NB_ECUDA, cudaGetErrorString(e));
    return NB_OK;
}

}  // extern "C"
