// nb_direct.cu -- direct-sum gravity (K1) and the compensated kick-drift (K7).
//
// Replaces BruteForceCPU::Exec/Update (src/Sim/BruteForceCPU.cpp:25-74) and
// the D3D11 pair BruteForceGPU + shaders/Compute/Gravity.csh, Update.csh
// (src/Sim/BruteForceGPU.cpp:45-71).
//
// Layout: bodies are float4 (x, y, z, m) in HBM, padded to a multiple of
// kPad with zero-mass bodies.  A work unit of K1 is (target block, source
// range): BLOCK*IPT target bodies held in registers against a contiguous
// range of source tiles.  Each 128-body source tile (2 KB) is moved from HBM
// to shared memory by the TMA engine (cp.async.bulk) into a double buffer
// guarded by mbarriers; every thread then reads each source body as a
// broadcast float4.  Forces are accumulated in FP32 in groups of kFold
// sources, and each group sum is folded into a Kahan-compensated total.
// Each unit writes its (sum, compensation) partials; K7 folds the partials of
// all source ranges in a fixed order (deterministic), applies G, and performs
// the kick-drift with Kahan-compensated velocity and position.
//
// Force law per source j on target i (reference law, Phys::Gravity,
// src/Sim/Physics.hpp:25-35, S = softening2):
//     a_i += m_j (p_j - p_i) / (r (r^2 + S)),   r = |p_j - p_i|
// evaluated with one MUFU.RSQ: 1/(r (r^2+S)) = rsqrt(r^2 (r^2+S)^2 + tiny).
// tiny = 1e-30 keeps the self pair (r = 0, dp = 0) finite, so it adds
// exactly zero; it is below the rounding of every real pair with S >= 1e-12.
// Plummer law: a_i += m_j (p_j - p_i) (r^2 + S)^{-3/2}.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include "nb_law.cuh"
#include <algorithm>
#include <cmath>

namespace nb {

// K1: grid (target blocks, source ranges). Writes part[split][i] (sum) and
// part[splits + split][i] (compensation).  polls bounds each wait for a
// source tile (kMaxPolls normally; smaller only to test the timeout path);
// the copies still in flight after a wait gave up are always waited for with
// the full budget before the block exits.  HEAVY: the state's largest mass
// may need more than the law's default self-pair guard (masses above 1e21);
// the guard is then read from *mmax, else it is the compile-time constant.
template <int LAW, int BLOCK, int IPT, bool COMP, bool HEAVY>
__global__ void __launch_bounds__(BLOCK) k_direct_force(const float4* __restrict__ pos, int n_pad,
                                                        int tiles_per_split, int ntiles, int splits, float S,
                                                        float4* __restrict__ part, int* __restrict__ err,
                                                        uint32_t polls, const unsigned* __restrict__ mmax) {
    __shared__ __align__(128) float4 tile[2][kTileJ];
    const float tiny = HEAVY ? self_pair_tiny(mmax) : kTiny;
    __shared__ __align__(8) uint64_t bar[2];

    const int split = blockIdx.y;
    const int ibase = blockIdx.x * BLOCK * IPT + threadIdx.x;

    float xi[IPT], yi[IPT], zi[IPT];
    float sx[IPT], sy[IPT], sz[IPT], cx[IPT], cy[IPT], cz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        float4 p = pos[ibase + k * BLOCK];
        xi[k] = p.x; yi[k] = p.y; zi[k] = p.z;
        sx[k] = sy[k] = sz[k] = 0.f;
        cx[k] = cy[k] = cz[k] = 0.f;
    }

    const int t_begin = split * tiles_per_split;
    const int nt = max(0, min(ntiles, t_begin + tiles_per_split) - t_begin);
    constexpr uint32_t kBytes = kTileJ * sizeof(float4);

    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < 2 && q < nt; ++q) {
            mbar_arrive_expect_tx(&bar[q], kBytes);
            bulk_g2s(tile[q], pos + (size_t)(t_begin + q) * kTileJ, kBytes, &bar[q]);
        }
    }

    int t = 0;
    bool abandoned = false;
    for (; t < nt; ++t) {
        const int b = t & 1;
        const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)((t >> 1) & 1), polls);
        const float4* tj = tile[b];
#pragma unroll 1
        for (int f = 0; f < kTileJ; f += kFold) {
            float tx[IPT], ty[IPT], tz[IPT];
            if constexpr (IPT % 2 == 0) {
                // Packed FP32x2: target bodies (2k, 2k+1) share every instruction.
                constexpr int P = IPT / 2;
                float2 ax[P], ay[P], az[P];
#pragma unroll
                for (int k = 0; k < P; ++k) ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);
                const float2 S2 = make_float2(S, S), T2 = make_float2(tiny, tiny);
#pragma unroll 4
                for (int j = 0; j < kFold; ++j) {
                    const float4 pj = tj[f + j];
                    const float2 jx = make_float2(pj.x, pj.x), jy = make_float2(pj.y, pj.y);
                    const float2 jz = make_float2(pj.z, pj.z), jm = make_float2(pj.w, pj.w);
#pragma unroll
                    for (int k = 0; k < P; ++k)
                        interact_x2<LAW>(jx, jy, jz, jm, make_float2(-xi[2 * k], -xi[2 * k + 1]),
                                         make_float2(-yi[2 * k], -yi[2 * k + 1]), make_float2(-zi[2 * k], -zi[2 * k + 1]),
                                         S2, T2, ax[k], ay[k], az[k]);
                }
#pragma unroll
                for (int k = 0; k < P; ++k) {
                    tx[2 * k] = ax[k].x; tx[2 * k + 1] = ax[k].y;
                    ty[2 * k] = ay[k].x; ty[2 * k + 1] = ay[k].y;
                    tz[2 * k] = az[k].x; tz[2 * k + 1] = az[k].y;
                }
            } else {
#pragma unroll
                for (int k = 0; k < IPT; ++k) tx[k] = ty[k] = tz[k] = 0.f;
#pragma unroll 4
                for (int j = 0; j < kFold; ++j) {
                    const float4 pj = tj[f + j];
#pragma unroll
                    for (int k = 0; k < IPT; ++k)
                        interact<LAW>(pj, xi[k], yi[k], zi[k], S, tiny, tx[k], ty[k], tz[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                if (COMP) {
                    kahan_add(sx[k], cx[k], tx[k]);
                    kahan_add(sy[k], cy[k], ty[k]);
                    kahan_add(sz[k], cz[k], tz[k]);
                } else {
                    sx[k] += tx[k]; sy[k] += ty[k]; sz[k] += tz[k];
                }
            }
        }
        // Every thread is done with tile[b]; agree on the wait outcome.
        if (__syncthreads_or(!ok)) { abandoned = true; break; }
        if (threadIdx.x == 0 && t + 2 < nt) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[b], kBytes);
            bulk_g2s(tile[b], pos + (size_t)(t_begin + t + 2) * kTileJ, kBytes, &bar[b]);
        }
    }
    if (abandoned) {
        // Let the copies still in flight land before the block's shared
        // memory is released (bounded), then report.
        if (threadIdx.x == 0) {
            for (int q = t; q < nt && q < t + 2; ++q)
                (void)mbar_wait_bounded(&bar[q & 1], (uint32_t)((q >> 1) & 1), kMaxPolls);
            record_error(err, DEV_WAIT_TIMEOUT);
        }
        return;
    }
    float4* psum = part + (size_t)split * n_pad;
    float4* pcmp = part + (size_t)(splits + split) * n_pad;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK;
        psum[i] = make_float4(sx[k], sy[k], sz[k], 0.f);
        pcmp[i] = make_float4(cx[k], cy[k], cz[k], 0.f);
    }
}

// K7: fold the partials of all source ranges (fixed order), apply G, add the
// pending initial forces, store the acceleration and, when update != 0,
// kick-drift: v += a dt; x += v dt / scale, both Kahan-compensated
// (src/Sim/BruteForceCPU.cpp:61-73).  When the error word is set (a force
// block abandoned a wait, or an earlier error has not been read yet) the
// step is abandoned: acceleration and state stay as they were.
// Render hand-off in the update's epilogue: the vertex (LWParticle layout,
// 32 bytes) of a body the update just moved, as two 16-byte stores.
__device__ __forceinline__ void write_vertex(nb_render_vertex* rv, const float4* rcol, float rscale, int i,
                                             const float4 x) {
    const float4 c = rcol[i];
    float4* o = reinterpret_cast<float4*>(rv + i);
    o[0] = make_float4(x.x, x.y, x.z, c.x);
    o[1] = make_float4(c.y, c.z, c.w, rscale);
}

// Body i's force from its source-split partials ([split][n_pad] sums, then
// [split][n_pad] compensations): compensated sum of the sums in split order,
// less the compensations.  The partials of 16 splits are loaded before they
// are added (in the same order), so that their loads overlap.
__device__ __forceinline__ float3 fold_partials(const float4* __restrict__ part, int splits, int n_pad, int i) {
    float ax = 0.f, ay = 0.f, az = 0.f, kx = 0.f, ky = 0.f, kz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
    auto add = [&](const float4 p, const float4 c) {
        kahan_add(ax, kx, p.x);
        kahan_add(ay, ky, p.y);
        kahan_add(az, kz, p.z);
        qx += c.x; qy += c.y; qz += c.z;
    };
    constexpr int kBatch = 16;
    int s = 0;
    for (; s + kBatch <= splits; s += kBatch) {
        float4 p[kBatch], c[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            p[u] = part[(size_t)(s + u) * n_pad + i];
            c[u] = part[(size_t)(splits + s + u) * n_pad + i];
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u) add(p[u], c[u]);
    }
    for (; s < splits; ++s) add(part[(size_t)s * n_pad + i], part[(size_t)(splits + s) * n_pad + i]);
    return make_float3(ax - (kx + qx), ay - (ky + qy), az - (kz + qz));
}

// kFoldLanes consecutive threads fold one body's partials: lane j takes
// splits j, j + kFoldLanes, ... (compensated, in that order), and the lanes'
// corrected sums are added by a butterfly (every lane gets the same total).
constexpr int kFoldLanes = 8;

__device__ __forceinline__ float3 fold_partials_lanes(const float4* __restrict__ part, int splits, int n_pad, int i,
                                                      int j) {
    float ax = 0.f, ay = 0.f, az = 0.f, kx = 0.f, ky = 0.f, kz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
    for (int s = j; s < splits; s += kFoldLanes) {
        const float4 p = part[(size_t)s * n_pad + i];
        const float4 c = part[(size_t)(splits + s) * n_pad + i];
        kahan_add(ax, kx, p.x);
        kahan_add(ay, ky, p.y);
        kahan_add(az, kz, p.z);
        qx += c.x; qy += c.y; qz += c.z;
    }
    float3 f = make_float3(ax - (kx + qx), ay - (ky + qy), az - (kz + qz));
#pragma unroll
    for (int o = 1; o < kFoldLanes; o <<= 1) {
        f.x += __shfl_xor_sync(0xffffffffu, f.x, o);
        f.y += __shfl_xor_sync(0xffffffffu, f.y, o);
        f.z += __shfl_xor_sync(0xffffffffu, f.z, o);
    }
    return f;
}

__global__ void k_direct_reduce_update(const float4* __restrict__ part, int splits, int n, int n_pad, float G,
                                       const float4* __restrict__ finit, float4* __restrict__ acc,
                                       float4* __restrict__ pos, float4* __restrict__ posc,
                                       float4* __restrict__ vel, float4* __restrict__ velc, float dt,
                                       float inv_scale, int update, int comp, nb_render_vertex* __restrict__ rv,
                                       const float4* __restrict__ rcol, float rscale,
                                       const int* __restrict__ err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / kFoldLanes, j = t % kFoldLanes;
    // whole groups of lanes leave together (n_pad bodies, a multiple of the block)
    if (i >= n_pad || *err != 0) return;
    const float3 f = fold_partials_lanes(part, splits, n_pad, i, j);
    if (i >= n || j != 0) return;
    float3 a = make_float3(G * f.x, G * f.y, G * f.z);
    if (finit) {
        const float4 f = finit[i];
        a.x += f.x; a.y += f.y; a.z += f.z;
    }
    acc[i] = make_float4(a.x, a.y, a.z, 0.f);
    if (!update) return;
    float4 v = vel[i], vc = velc[i], x = pos[i], xc = posc[i];
    if (comp) {
        kahan_add(v.x, vc.x, a.x * dt);
        kahan_add(v.y, vc.y, a.y * dt);
        kahan_add(v.z, vc.z, a.z * dt);
        kahan_add(x.x, xc.x, ((v.x - vc.x) * dt) * inv_scale);
        kahan_add(x.y, xc.y, ((v.y - vc.y) * dt) * inv_scale);
        kahan_add(x.z, xc.z, ((v.z - vc.z) * dt) * inv_scale);
        velc[i] = vc;
        posc[i] = xc;
    } else {
        v.x += a.x * dt; v.y += a.y * dt; v.z += a.z * dt;
        x.x += (v.x * dt) * inv_scale; x.y += (v.y * dt) * inv_scale; x.z += (v.z * dt) * inv_scale;
    }
    vel[i] = v;
    pos[i] = x;
    if (rv) write_vertex(rv, rcol, rscale, i, x);
}

// Kick-drift from a stored acceleration (Barnes-Hut path,
// src/Sim/BarnesHut.cpp:81-95).
__global__ void k_kick_drift(const float4* __restrict__ acc, int n, float4* __restrict__ pos,
                             float4* __restrict__ posc, float4* __restrict__ vel, float4* __restrict__ velc,
                             float dt, float inv_scale, int comp, nb_render_vertex* __restrict__ rv,
                             const float4* __restrict__ rcol, float rscale, const int32_t* __restrict__ hold,
                             int int_cap, int cell_cap, int* __restrict__ held) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (hold && !tree_fits(hold, int_cap, cell_cap)) {   // the step is held: the state stays as it was
        if (i == 0) atomicAdd(held, 1);
        return;
    }
    const float4 a = acc[i];
    float4 v = vel[i], vc = velc[i], x = pos[i], xc = posc[i];
    if (comp) {
        kahan_add(v.x, vc.x, a.x * dt);
        kahan_add(v.y, vc.y, a.y * dt);
        kahan_add(v.z, vc.z, a.z * dt);
        kahan_add(x.x, xc.x, ((v.x - vc.x) * dt) * inv_scale);
        kahan_add(x.y, xc.y, ((v.y - vc.y) * dt) * inv_scale);
        kahan_add(x.z, xc.z, ((v.z - vc.z) * dt) * inv_scale);
        velc[i] = vc;
        posc[i] = xc;
    } else {
        v.x += a.x * dt; v.y += a.y * dt; v.z += a.z * dt;
        x.x += (v.x * dt) * inv_scale; x.y += (v.y * dt) * inv_scale; x.z += (v.z * dt) * inv_scale;
    }
    vel[i] = v;
    pos[i] = x;
    if (rv) write_vertex(rv, rcol, rscale, i, x);
}

namespace {

template <int LAW, int BLOCK, int IPT, bool COMP>
void launch_force_t(dim3 grid, cudaStream_t st, const float4* pos, int n_pad, int tps, int ntiles, int splits,
                    float S, float4* part, int* err, uint32_t polls, const unsigned* mmax, bool heavy) {
    if (heavy)
        k_direct_force<LAW, BLOCK, IPT, COMP, true><<<grid, BLOCK, 0, st>>>(pos, n_pad, tps, ntiles, splits, S, part,
                                                                           err, polls, mmax);
    else
        k_direct_force<LAW, BLOCK, IPT, COMP, false><<<grid, BLOCK, 0, st>>>(pos, n_pad, tps, ntiles, splits, S,
                                                                            part, err, polls, mmax);
}

template <int LAW, bool COMP>
bool launch_force_law(int block, int ipt, dim3 grid, cudaStream_t st, const float4* pos, int n_pad, int tps,
                      int ntiles, int splits, float S, float4* part, int* err, uint32_t polls,
                      const unsigned* mmax, bool heavy) {
#define NB_CASE(B, I)                                                                                    \
    if (block == B && ipt == I) {                                                                        \
        launch_force_t<LAW, B, I, COMP>(grid, st, pos, n_pad, tps, ntiles, splits, S, part, err, polls, mmax, heavy); \
        return true;                                                                                     \
    }
    NB_CASE(64, 1) NB_CASE(64, 2) NB_CASE(64, 4) NB_CASE(64, 8)
    NB_CASE(128, 1) NB_CASE(128, 2) NB_CASE(128, 4) NB_CASE(128, 8)
    NB_CASE(256, 1) NB_CASE(256, 2) NB_CASE(256, 4)
#undef NB_CASE
    return false;
}

}  // namespace

int direct_splits(const nb_sim* sim, const DirectTuning& t, size_t n_pad) {
    const int ntiles = (int)(n_pad / kTileJ);
    const int iblocks = (int)(n_pad / (size_t)(t.block * t.ipt));
    int splits = t.splits;
    if (splits <= 0) {
        const int target = std::max(1, sim->sm_count) * 256;  // many short units: dynamic balance
        splits = (target + iblocks - 1) / iblocks;
        // keep the partials (2 float4 per body per split) within 512 MB
        const size_t cap = (512ull << 20) / (n_pad * 2 * sizeof(float4));
        splits = (int)std::min<size_t>((size_t)splits, std::max<size_t>(1, cap));
    }
    splits = std::max(1, std::min(splits, ntiles));
    const int tps = (ntiles + splits - 1) / splits;
    return (ntiles + tps - 1) / tps;
}

size_t direct_part_entries(const nb_sim* sim, const DirectTuning& t, size_t n_pad) {
    return (size_t)direct_splits(sim, t, n_pad) * 2 * n_pad;
}

static DirectTuning default_tuning(size_t n_pad) {
    DirectTuning t;
    t.block = 128;
    t.ipt = n_pad >= 16384 ? 2 : 1;
    return t;
}

cudaError_t direct_force_update(nb_sim* sim, float dt, bool update) {
    DirectTuning t = sim->tune;
    if (!sim->tune_set) {
        t = default_tuning(sim->n_pad);
        t.splits = sim->tune.splits;
    }
    if (t.block <= 0 || t.ipt <= 0) t = default_tuning(sim->n_pad);
    // A tuning whose target block does not divide the padded size falls back.
    if (sim->n_pad % (size_t)(t.block * t.ipt) != 0) t = default_tuning(sim->n_pad);
    const int splits = direct_splits(sim, t, sim->n_pad);
    const size_t need = (size_t)splits * 2 * sim->n_pad;
    if (need > sim->part_cap) {
        dev_free(sim->part, sim->stream);
        sim->part = nullptr;
        sim->part_cap = 0;
        cudaError_t e = dev_alloc(&sim->part, need * sizeof(float4));
        if (e != cudaSuccess) return e;
        sim->part_cap = need;
    }
    const int ntiles = (int)(sim->n_pad / kTileJ);
    const int tps = (ntiles + splits - 1) / splits;
    dim3 grid((unsigned)(sim->n_pad / (size_t)(t.block * t.ipt)), (unsigned)splits);
    const float S = (float)sim->prm.softening2;
    const bool comp = !(sim->prm.flags & NB_FLAG_NO_COMPENSATION);
    bool ok;
    {
    PhaseScope ps(sim, 0);
    if (sim->prm.law == NB_LAW_PLUMMER)
        ok = comp ? launch_force_law<NB_LAW_PLUMMER, true>(t.block, t.ipt, grid, sim->stream, sim->pos,
                                                          (int)sim->n_pad, tps, ntiles, splits, S, sim->part,
                                                          sim->d_err, sim->wait_polls, sim->d_mmax, sim->heavy)
                  : launch_force_law<NB_LAW_PLUMMER, false>(t.block, t.ipt, grid, sim->stream, sim->pos,
                                                           (int)sim->n_pad, tps, ntiles, splits, S, sim->part,
                                                           sim->d_err, sim->wait_polls, sim->d_mmax, sim->heavy);
    else
        ok = comp ? launch_force_law<NB_LAW_REFERENCE, true>(t.block, t.ipt, grid, sim->stream, sim->pos,
                                                            (int)sim->n_pad, tps, ntiles, splits, S, sim->part,
                                                            sim->d_err, sim->wait_polls, sim->d_mmax, sim->heavy)
                  : launch_force_law<NB_LAW_REFERENCE, false>(t.block, t.ipt, grid, sim->stream, sim->pos,
                                                             (int)sim->n_pad, tps, ntiles, splits, S, sim->part,
                                                             sim->d_err, sim->wait_polls, sim->d_mmax, sim->heavy);
    }
    if (!ok) return cudaErrorInvalidConfiguration;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int n = (int)sim->n;
    const float inv_scale = (float)(1.0 / sim->prm.pos_scale);
    PhaseScope ps(sim, 1);
    static_assert(kPad % (256 / kFoldLanes) == 0, "the fold's blocks cover whole padded bodies");
    k_direct_reduce_update<<<(unsigned)(sim->n_pad * kFoldLanes / 256), 256, 0, sim->stream>>>(
        sim->part, splits, n, (int)sim->n_pad, (float)sim->prm.G, sim->finit_pending ? sim->finit : nullptr,
        sim->acc, sim->pos, sim->posc, sim->vel, sim->velc, dt, inv_scale, update ? 1 : 0, comp ? 1 : 0,
        update ? sim->render : nullptr, sim->rcolour, sim->rscale, sim->d_err);
    sim->finit_pending = false;
    const double nn = (double)sim->n;
    sim->inter_last = (uint64_t)(nn * (nn - 1.0));
    return cudaGetLastError();
}

cudaError_t kick_drift(nb_sim* sim, float dt, const int32_t* hold, int int_cap, int cell_cap, int* held) {
    const int n = (int)sim->n;
    const bool comp = !(sim->prm.flags & NB_FLAG_NO_COMPENSATION);
    PhaseScope ps(sim, 7);
    k_kick_drift<<<(n + 255) / 256, 256, 0, sim->stream>>>(sim->acc, n, sim->pos, sim->posc, sim->vel, sim->velc,
                                                           dt, (float)(1.0 / sim->prm.pos_scale), comp ? 1 : 0,
                                                           sim->render, sim->rcolour, sim->rscale, hold, int_cap,
                                                           cell_cap, held);
    return cudaGetLastError();
}

}  // namespace nb

// ---------------------------------------------------------------------------
// Allocation-free direct-sum accelerations.
//
// For callers that must not allocate device memory while they step: a render
// loop that stays inside a fixed device-memory budget, a host that hands in
// buffers owned by its own allocator, or a thread that must not block (every
// cudaFree synchronises the whole device).  The caller passes device input
// and output buffers; the working memory of the kernels is a file-scope
// __device__ array of fixed size that every GPU loading this library holds
// until the process exits.  It has no counterpart in the reference.
// ---------------------------------------------------------------------------
#include <mutex>

namespace nb {

constexpr int kNoAllocMaxSplits = 8;
// padded copy of the input + (sum, compensation) partials of up to 8 source ranges
constexpr size_t kNoAllocScratch = (size_t)NB_NOALLOC_MAX_BODIES * (1 + 2 * kNoAllocMaxSplits);
static __device__ __align__(256) float4 g_noalloc_scratch[kNoAllocScratch];   // 17.8 MB
static __device__ int g_noalloc_err;
// float bits of the call's largest |mass| (the force law's self-pair guard);
// zero between calls: the reduce kernel clears it after the force kernel read it
static __device__ unsigned g_noalloc_mmax;

// Copies n bodies into the scratch and zero-fills the padding (zero-mass
// bodies at the origin contribute exactly nothing); clears the error word and
// records the largest |mass|.
__global__ void k_noalloc_stage(const float4* __restrict__ in, int n, int n_pad, float4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) g_noalloc_err = 0;
    if (i < n_pad) {
        const float4 p = i < n ? in[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        out[i] = p;
        if (i < n) atomicMax(&g_noalloc_mmax, __float_as_uint(fabsf(p.w)));
    }
}

// Folds the partials like k_direct_reduce_update; a force kernel whose bounded
// wait ran out poisons the output with NaN, since nothing is read back.
__global__ void k_noalloc_reduce(const float4* __restrict__ part, int splits, int n, int n_pad, float G,
                                 float4* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 f = fold_partials(part, splits, n_pad, i);
    float4 a = make_float4(G * f.x, G * f.y, G * f.z, 0.f);
    if (g_noalloc_err != 0) a = make_float4(NAN, NAN, NAN, NAN);
    acc[i] = a;
    if (i == 0) g_noalloc_mmax = 0u;
}

namespace {
std::mutex g_noalloc_mu;
float4* g_noalloc_ptr[256] = {};   // device address of the scratch, per device ordinal
int* g_noalloc_err_ptr[256] = {};
unsigned* g_noalloc_mmax_ptr[256] = {};
}  // namespace

}  // namespace nb

extern "C" int nb_direct_accel_noalloc(const float* pos_mass4, size_t n, float* accel4, double G, double softening2,
                                       int law, void* stream) {
    using namespace nb;
    if (!pos_mass4 || !accel4 || n == 0) return NB_EINVAL;
    if (n > (size_t)NB_NOALLOC_MAX_BODIES) return NB_EINVAL;
    if (law != NB_LAW_REFERENCE && law != NB_LAW_PLUMMER) return NB_EINVAL;
    if (!std::isfinite(G) || !std::isfinite(softening2) || softening2 < 0 ||
        (law == NB_LAW_PLUMMER && softening2 <= 0))
        return NB_EINVAL;
    if ((reinterpret_cast<uintptr_t>(pos_mass4) | reinterpret_cast<uintptr_t>(accel4)) & 15u) return NB_EINVAL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) { cudaGetLastError(); return NB_ECUDA; }
    float4* scratch = nullptr;
    int* err = nullptr;
    unsigned* mmax = nullptr;
    {
        // Set-up on the first call on each device, with that device current.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            void* q = nullptr;
            void* r = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess ||
                cudaGetSymbolAddress(&q, g_noalloc_err) != cudaSuccess ||
                cudaGetSymbolAddress(&r, g_noalloc_mmax) != cudaSuccess || !p || !q || !r) {
                cudaGetLastError();
                return NB_ECUDA;
            }
            g_noalloc_ptr[dev] = static_cast<float4*>(p);
            g_noalloc_err_ptr[dev] = static_cast<int*>(q);
            g_noalloc_mmax_ptr[dev] = static_cast<unsigned*>(r);
        }
        scratch = g_noalloc_ptr[dev];
        err = g_noalloc_err_ptr[dev];
        mmax = g_noalloc_mmax_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n_pad = pad_up(n, kPad);
    const int ntiles = (int)(n_pad / kTileJ);
    int splits = std::min(kNoAllocMaxSplits, ntiles);
    const int tps = (ntiles + splits - 1) / splits;
    splits = (ntiles + tps - 1) / tps;
    float4* pos = scratch;
    float4* part = scratch + n_pad;
    k_noalloc_stage<<<(unsigned)((n_pad + 255) / 256), 256, 0, st>>>(reinterpret_cast<const float4*>(pos_mass4),
                                                                    (int)n, (int)n_pad, pos);
    const int block = 128, ipt = n_pad >= 16384 ? 2 : 1;
    dim3 grid((unsigned)(n_pad / (size_t)(block * ipt)), (unsigned)splits);
    const float S = (float)softening2;
    bool ok = law == NB_LAW_PLUMMER
                  ? launch_force_law<NB_LAW_PLUMMER, true>(block, ipt, grid, st, pos, (int)n_pad, tps, ntiles, splits,
                                                          S, part, err, kMaxPolls, mmax, true)
                  : launch_force_law<NB_LAW_REFERENCE, true>(block, ipt, grid, st, pos, (int)n_pad, tps, ntiles,
                                                            splits, S, part, err, kMaxPolls, mmax, true);
    if (!ok) return NB_EINVAL;
    k_noalloc_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, splits, (int)n, (int)n_pad, (float)G,
                                                                 reinterpret_cast<float4*>(accel4));
    if (cudaGetLastError() != cudaSuccess) return NB_ECUDA;
    return NB_OK;
}
