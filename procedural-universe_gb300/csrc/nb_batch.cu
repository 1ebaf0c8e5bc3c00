// nb_batch.cu -- batched form: many independent galaxies stepped together,
// one launch per phase, the whole step replayed from a captured CUDA graph,
// launch parameters chosen by the project's autotuner.  Kernels: see
// nb_batch_kernels.cuh.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include "nb_law.cuh"
#include "nb_batch_kernels.cuh"
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

using namespace nb;

struct nb_batch {
    nb_params base{};
    size_t bh_threshold = 8192;
    double bh_theta = 0.6;
    // Far field of the group traversal (a third-order local expansion at the
    // group's centre, evaluated once per body).  An accepted cell joins it
    //  - relative rule, once the group's bodies have accelerations from an
    //    earlier evaluation: when the cell's truncation-error estimate
    //    m / r^2 (r_g / r)^4 (r its distance from the centre, r_g the group's
    //    half-diagonal) is below far_alpha times the group's smallest |a| / G
    //    and r_g / r < far_cap;
    //  - geometric rule otherwise (first evaluation of a state, far_alpha 0):
    //    when r_g / r < far_eta.
    // far_eta 0 and far_alpha 0 evaluate every accepted cell per body.
    double far_eta = kFarEta;
    double far_alpha = kFarAlpha;
    double far_cap = kFarCap;
    nb_sim* core = nullptr;   // device state of all bodies, stream, error word, tree buffers
    std::string err;
    // galaxies as added
    struct Gal {
        size_t n = 0;
        bool bh = false;
        size_t off = 0;   // first body in the concatenated arrays
        int idx = -1;     // slot (Barnes-Hut) or direct-galaxy index
        size_t n_pad = 0;
        const float4* dsrc[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // device source (pos, posc, vel, velc, acc)
        int gen_model = -1;      // >= 0: generated on the device at commit (nb_batch_add_generated)
        uint64_t gen_seed = 0;
    };
    std::vector<Gal> gal;
    std::vector<std::vector<float>> h_pos, h_vel;
    bool committed = false;
    size_t n_bh = 0, dir_begin = 0, n_total = 0, n_real = 0;
    int nslot = 0, ndgal = 0;
    // Barnes-Hut tables
    int32_t* body_slot = nullptr;
    int4* gal_range = nullptr;
    float4* gal_box = nullptr;
    int32_t* gal_root = nullptr;
    int32_t* slot_start = nullptr;
    int4* groups = nullptr;          // traversal groups, rebuilt on the device every step
    int group_cap = 0;
    int* group_ctr = nullptr;        // [0] groups emitted, [1] next group to traverse
    unsigned* box_bits = nullptr;    // 6 ordered words per galaxy: min xyz, max xyz
    CellRec* cell_rec = nullptr;    // per cell: centre of mass, walk record, quadrupole (nb_cellrec.cuh)
    size_t qcap = 0;
    // direct-sum tables
    int32_t* body_dgal = nullptr;
    int4* dgal = nullptr;
    int4* units = nullptr;
    int32_t* unit_comp = nullptr;
    int nunits = 0;
    float4* part = nullptr;
    size_t part_cap = 0;
    int* next_unit = nullptr;
    uint64_t direct_pairs = 0;
    // steps whose octree did not fit its arrays leave the state unchanged and
    // count here; the wait resizes the tree and runs them again
    int* held = nullptr;
    float pending_dt = 0.f;
    int steps_not_run = 0;   // of the last launch, when batch_wait gave up (NB_ENOMEM)
    // tuning and graph
    nb_tuning tune{128, 1, 1024, 16, 128};
    cudaGraphExec_t exec = nullptr;
    float graph_dt = NAN;
    bool graph_dirty = true;
    uint64_t graph_kernels = 0;
};

namespace {

int bfail(nb_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

#define NB_BCUDA(b, call)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return bfail((b), NB_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src, cudaStream_t st) {
    dev_free(*dst, st);
    *dst = nullptr;
    if (src.empty()) return cudaSuccess;
    cudaError_t e = dev_alloc(dst, src.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

bool tuning_valid(const nb_tuning& t) {
    const bool blk = t.direct_block == 64 || t.direct_block == 128 || t.direct_block == 256;
    const bool ipt = t.direct_ipt == 1 || t.direct_ipt == 2;
    return blk && ipt && t.direct_block * t.direct_ipt <= 256 && t.direct_jtile >= 128 && t.direct_jtile % 128 == 0 && t.leaf_size >= 1 &&
           t.leaf_size <= 64 && t.traverse_block == 128;
}

// Work units of the direct-sum galaxies for the current tuning.
int plan_units(nb_batch* b) {
    std::vector<int4> units, dg(b->ndgal);
    std::vector<int32_t> ucomp;
    const int tb = b->tune.direct_block * b->tune.direct_ipt;
    const int utiles = b->tune.direct_jtile / kDirTile;
    size_t part_base = 0;
    for (const auto& g : b->gal) {
        if (g.bh) continue;
        const int ntiles = (int)(g.n_pad / kDirTile);
        const int splits = (ntiles + utiles - 1) / utiles;
        dg[g.idx] = make_int4((int)g.off, (int)g.n_pad, splits, (int)part_base);
        const int comp = splits * (int)g.n_pad;
        for (int blk = 0; blk < (int)(g.n_pad / tb); ++blk)
            for (int s = 0; s < splits; ++s) {
                const int t0 = s * utiles;
                const int nt = std::min(utiles, ntiles - t0);
                units.push_back(make_int4((int)g.off + blk * tb, (int)(g.off / kDirTile) + t0, nt,
                                          (int)part_base + s * (int)g.n_pad + blk * tb));
                ucomp.push_back(comp);
            }
        part_base += 2 * (size_t)splits * g.n_pad;
    }
    if (part_base > (size_t)INT32_MAX) return bfail(b, NB_ENOMEM, "direct-sum partials exceed 2^31 entries");
    NB_BCUDA(b, upload(&b->units, units, b->core->stream));
    NB_BCUDA(b, upload(&b->unit_comp, ucomp, b->core->stream));
    NB_BCUDA(b, upload(&b->dgal, dg, b->core->stream));
    b->nunits = (int)units.size();
    if (part_base > b->part_cap) {
        dev_free(b->part, b->core->stream);
        b->part = nullptr;
        b->part_cap = 0;
        NB_BCUDA(b, dev_alloc(&b->part, std::max<size_t>(part_base, 1) * sizeof(float4)));
        b->part_cap = part_base;
    }
    b->graph_dirty = true;
    return NB_OK;
}

template <int LAW>
bool launch_direct_t(nb_batch* b, int grid, cudaStream_t st, float S) {
    const int blk = b->tune.direct_block, ipt = b->tune.direct_ipt;
#define NB_BD(B, I)                                                                                           \
    if (blk == B && ipt == I) {                                                                               \
        k_batch_direct<LAW, B, I><<<grid, B, 0, st>>>(b->core->pos, b->units, b->unit_comp, b->nunits,         \
                                                      b->next_unit, S, b->core->d_mmax, b->part);             \
        return true;                                                                                          \
    }
    NB_BD(64, 1) NB_BD(64, 2) NB_BD(128, 1) NB_BD(128, 2) NB_BD(256, 1)
#undef NB_BD
    return false;
}

// One step (update) or one force evaluation (no update) of every galaxy,
// enqueued on the core stream without host synchronisation; tree_only stops
// once the octree's node counts are known (no node written).
int enqueue_step(nb_batch* b, float dt, bool update, bool tree_only = false) {
    nb_sim* c = b->core;
    cudaStream_t st = c->stream;
    const float S = (float)b->base.softening2;
    const float G = (float)b->base.G;
    TreeBuffers& t = c->tree;
    if (b->n_bh > 0) {
        const int n = (int)b->n_bh;
        {
            // the step's counters, the galaxy cubes, then the forest's keys with the sort's histograms
            PhaseScope ps(c, NB_PHASE_KEYS, 2);
            const int words = std::max(6 * b->nslot, tree_counter_words());
            k_gal_box_init<<<(words + 255) / 256, 256, 0, st>>>(b->box_bits, b->nslot, t.counters,
                                                               tree_counter_words(), n, t.interactions, b->group_ctr,
                                                               b->ndgal > 0 ? b->next_unit : nullptr);
            k_gal_box_chunks<<<(unsigned)((n + kBoxChunk - 1) / kBoxChunk), 256, 0, st>>>(c->pos, b->body_slot, n,
                                                                                       b->nslot, b->box_bits);
        }
        NB_BCUDA(b, tree_batch_keys(c, c->pos, b->body_slot, n, b->box_bits, b->nslot, b->gal_box));
        NB_BCUDA(b, tree_build_graph(c, c->pos, n, kBatchDepth, tree_only, b->cell_rec));
        if (tree_only) return NB_OK;
        {
            PhaseScope ps(c, NB_PHASE_MASS, 3);
            k_batch_moments<<<(unsigned)((t.int_cap + 255) / 256), 256, 0, st>>>(
                (int)t.int_cap, t.counters, t.int_parent, t.int_nint, t.int_pending, t.int_cell, t.int_block,
                t.int_mask, t.int_first, t.int_level, b->cell_rec, (int)t.cell_cap, c->d_err);
            k_batch_roots<<<(b->nslot + 127) / 128, 128, 0, st>>>(b->slot_start, b->nslot, t.keys[0], t.pos_nint,
                                                                 t.int_cell, t.counters, (int)t.int_cap,
                                                                 (int)t.cell_cap, b->gal_root, c->d_err);
            k_batch_groups<<<(unsigned)((t.int_cap + 255) / 256), 256, 0, st>>>(
                (int)t.int_cap, t.counters, t.int_cell, b->cell_rec,
                t.vals[0], b->body_slot, (int)t.cell_cap, n, b->groups, b->group_cap, b->group_ctr, c->d_err);
        }
        {
            PhaseScope ps(c, NB_PHASE_TRAVERSE);
            const float th = (float)b->bh_theta;
            // persistent: as many warps as fit on the GPU, groups taken from the queue
            int occ = 1;
            if (b->base.law == NB_LAW_PLUMMER)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_group_traverse<NB_LAW_PLUMMER>, kGWarps * 32, 0);
            else
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_group_traverse<NB_LAW_REFERENCE>, kGWarps * 32, 0);
            const int max_blocks = (b->group_cap + kGWarps - 1) / kGWarps;
            const int blocks = std::max(1, std::min(max_blocks, c->sm_count * std::max(1, occ)));
#define NB_GT(L)                                                                                                  \
    k_group_traverse<L><<<blocks, kGWarps * 32, 0, st>>>(                                                         \
        b->groups, b->group_ctr, b->group_cap, b->group_ctr + 1, t.spos, t.vals[0], b->cell_rec, b->gal_box,      \
        b->gal_root, b->nslot,                                                                                    \
        (int)t.cell_cap, n, (int)t.int_cap, b->tune.leaf_size, th * th, S, G, (float)(b->far_eta * b->far_eta),   \
        (float)(b->far_alpha / b->base.G), (float)(b->far_cap * b->far_cap),                                      \
        100.f * S, c->d_mmax, c->acc, t.interactions, c->d_err)
            if (b->base.law == NB_LAW_PLUMMER) NB_GT(NB_LAW_PLUMMER);
            else NB_GT(NB_LAW_REFERENCE);
#undef NB_GT
        }
        NB_BCUDA(b, cudaGetLastError());
    }
    if (b->ndgal > 0) {
        PhaseScope ps(c, NB_PHASE_DIRECT_FORCE, 2);
        if (b->n_bh == 0) NB_BCUDA(b, cudaMemsetAsync(b->next_unit, 0, sizeof(int), st));   // else cleared with the counters
        int occ = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_direct<NB_LAW_REFERENCE, 128, 1>,
                                                      b->tune.direct_block, 0);
        const int grid = std::max(1, std::min(b->nunits, c->sm_count * std::max(1, occ)));
        const bool ok = b->base.law == NB_LAW_PLUMMER ? launch_direct_t<NB_LAW_PLUMMER>(b, grid, st, S)
                                                      : launch_direct_t<NB_LAW_REFERENCE>(b, grid, st, S);
        if (!ok) return bfail(b, NB_EINVAL, "unsupported direct tuning");
        const int cnt = (int)(b->n_total - b->dir_begin);
        k_batch_direct_reduce<<<(cnt + 255) / 256, 256, 0, st>>>(b->body_dgal, b->dgal, (int)b->dir_begin, cnt, G,
                                                                b->part, c->acc);
        NB_BCUDA(b, cudaGetLastError());
    }
    if (update) {
        NB_BCUDA(b, kick_drift(c, dt, b->n_bh > 0 ? t.counters : nullptr, (int)t.int_cap, (int)t.cell_cap, b->held));
    }
    return NB_OK;
}

int read_tree_counts(nb_batch* b, int32_t* h) {
    NB_BCUDA(b, cudaMemcpyAsync(h, b->core->tree.counters, TC_COUNT * 4, cudaMemcpyDeviceToHost, b->core->stream));
    NB_BCUDA(b, cudaStreamSynchronize(b->core->stream));
    return NB_OK;
}

int reserve_tree(nb_batch* b, size_t n_int, size_t n_cells) {
    if (b->n_bh == 0) return NB_OK;
    NB_BCUDA(b, tree_reserve_graph(b->core, (int)b->n_bh, n_int, n_cells));
    const size_t cap = b->core->tree.cell_cap;
    if (cap > b->qcap) {
        dev_free(b->cell_rec, b->core->stream);
        b->cell_rec = nullptr;
        NB_BCUDA(b, dev_alloc(&b->cell_rec, cap * sizeof(CellRec)));
        b->qcap = cap;
    }
    b->graph_dirty = true;
    return NB_OK;
}

// Sizes the tree capacity from measured counts (a synchronising force pass).
int size_tree(nb_batch* b) {
    if (b->n_bh == 0) return NB_OK;
    // the counting pass writes no node: the node arrays need no room yet
    int rc = reserve_tree(b, 1, 1);
    if (rc) return rc;
    rc = enqueue_step(b, 0.f, false, true);
    if (rc) return rc;
    int32_t h[TC_COUNT];
    rc = read_tree_counts(b, h);
    if (rc) return rc;
    const size_t ni = (size_t)h[TC_NINT], nc = (size_t)h[TC_NINT] + (size_t)h[TC_NLEAF];
    // the traversal's stack entries carry a cell index below kStackCellLimit
    if (nc >= (size_t)kStackCellLimit)
        return bfail(b, NB_EINVAL, "batch too large: its octree needs more than 2^27 cells (about 10^8 "
                                   "Barnes-Hut bodies); split it over several batches");
    // room for the tree to grow as the galaxies evolve
    return reserve_tree(b, 2 * ni + 64, 2 * nc + 64);
}

int build_graph(nb_batch* b, float dt) {
    nb_sim* c = b->core;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    const bool prof = c->prof.on;
    c->prof.on = false;
    const uint64_t l0 = c->prof.launches;
    NB_BCUDA(b, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_step(b, dt, true);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->prof.on = prof;
    b->graph_kernels = c->prof.launches - l0;
    c->prof.launches = l0;
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return bfail(b, NB_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, NB_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    b->graph_dt = dt;
    b->graph_dirty = false;
    return NB_OK;
}

// Host side of tree_fits: the counts of the last build against the capacities.
bool tree_counts_fit(const nb_batch* b, const int32_t* h) {
    const TreeBuffers& t = b->core->tree;
    return h[TC_OVERFLOW] == 0 && h[TC_HASHFAIL] == 0 && (size_t)h[TC_NINT] <= t.int_cap &&
           (size_t)h[TC_NINT] + (size_t)h[TC_NLEAF] <= t.cell_cap;
}

// Waits for the stream; *fits (if given) receives whether the last octree
// fitted its arrays, otherwise a tree that did not is an error.
int sync_check(nb_batch* b, bool* fits = nullptr) {
    int rc = nb_synchronize(b->core);
    if (rc) return bfail(b, rc, nb_last_error(b->core));
    if (fits) *fits = true;
    if (b->n_bh > 0) {
        int32_t h[TC_COUNT];
        rc = read_tree_counts(b, h);
        if (rc) return rc;
        if (!tree_counts_fit(b, h)) {
            if (fits) *fits = false;
            else return bfail(b, NB_ENOMEM, "the batched octree outgrew its arrays");
        }
    }
    return NB_OK;
}

const nb_batch::Gal* find(nb_batch* b, int32_t galaxy) {
    if (galaxy < 0 || (size_t)galaxy >= b->gal.size()) return nullptr;
    return &b->gal[(size_t)galaxy];
}

}  // namespace

// ---- device-side hand-over between batches (used by the served form) -------
namespace nb {

// Adds a galaxy whose state (position+mass, position compensation, velocity,
// velocity compensation) lives in device memory, e.g. in another batch; the
// source must stay valid until nb_batch_commit returns.
int batch_add_device(nb_batch* b, const float4* pos, const float4* posc, const float4* vel, const float4* velc,
                     const float4* acc, size_t n, int32_t* galaxy) {
    if (!b || !pos || !posc || !vel || !velc || !acc || n == 0) return NB_EINVAL;
    if (b->committed) return bfail(b, NB_EBADSTATE, "galaxies are added before nb_batch_commit");
    if (n > kMaxGalaxyBodies) return bfail(b, NB_EINVAL, "galaxy too large for the batched form");
    b->h_pos.emplace_back();
    b->h_vel.emplace_back();
    nb_batch::Gal g;
    g.n = n;
    g.bh = n >= b->bh_threshold;
    g.dsrc[0] = pos; g.dsrc[1] = posc; g.dsrc[2] = vel; g.dsrc[3] = velc; g.dsrc[4] = acc;
    b->gal.push_back(g);
    if (galaxy) *galaxy = (int32_t)(b->gal.size() - 1);
    return NB_OK;
}

// Device state of a committed galaxy.
int batch_device_state(nb_batch* b, int32_t galaxy, const float4** pos, const float4** posc, const float4** vel,
                       const float4** velc, const float4** acc, size_t* n) {
    if (!b || !b->committed || galaxy < 0 || (size_t)galaxy >= b->gal.size()) return NB_EINVAL;
    const auto& g = b->gal[(size_t)galaxy];
    *pos = b->core->pos + g.off;
    *posc = b->core->posc + g.off;
    *vel = b->core->vel + g.off;
    *velc = b->core->velc + g.off;
    *acc = b->core->acc + g.off;
    *n = g.n;
    return NB_OK;
}

int batch_set_tuning_quiet(nb_batch* b, const nb_tuning& t) { return nb_batch_set_tuning(b, &t); }

int batch_launch_steps(nb_batch* b, float dt, int nsteps) {
    if (!b) return NB_EINVAL;
    if (!b->committed) return bfail(b, NB_EBADSTATE, "nb_batch_commit first");
    if (nsteps < 0 || !std::isfinite(dt)) return bfail(b, NB_EINVAL, "bad dt or nsteps");
    cudaSetDevice(b->core->dev);
    if (b->graph_dirty || !(b->graph_dt == dt) || !b->exec) {
        int rc = build_graph(b, dt);
        if (rc) return rc;
    }
    NB_BCUDA(b, cudaMemsetAsync(b->held, 0, sizeof(int), b->core->stream));
    b->pending_dt = dt;
    for (int k = 0; k < nsteps; ++k) {
        NB_BCUDA(b, cudaGraphLaunch(b->exec, b->core->stream));
        b->core->prof.launches += b->graph_kernels;
    }
    return NB_OK;
}

// Steps held because the octree outgrew its arrays (positions evolved, or a
// new state was written) are the last ones of the launch: the tree is sized
// again from the current state and they run once more.
int batch_wait(nb_batch* b) {
    if (!b) return NB_EINVAL;
    cudaSetDevice(b->core->dev);
    b->steps_not_run = 0;
    for (int attempt = 0;; ++attempt) {
        int rc = nb_synchronize(b->core);
        if (rc) return bfail(b, rc, nb_last_error(b->core));
        int held = 0;
        NB_BCUDA(b, cudaMemcpy(&held, b->held, sizeof(int), cudaMemcpyDeviceToHost));
        if (held == 0) return sync_check(b);
        if (attempt == 3) {
            // the held steps are the last ones of the launch and left the state as it was
            b->steps_not_run = held;
            return bfail(b, NB_ENOMEM, "the batched octree kept outgrowing its arrays");
        }
        rc = size_tree(b);
        if (rc) return rc;
        rc = batch_launch_steps(b, b->pending_dt, held);
        if (rc) return rc;
    }
}

int batch_steps_not_run(const nb_batch* b) { return b ? b->steps_not_run : 0; }

}  // namespace nb

extern "C" {

int nb_batch_create(const nb_params* base, size_t bh_threshold, double bh_theta, nb_batch** out) {
    try {
        if (!base || !out) return NB_EINVAL;
        *out = nullptr;
        if (!(bh_theta > 0) || !std::isfinite(bh_theta) || bh_threshold < 2) return NB_EINVAL;
        nb_params p = *base;
        p.kind = NB_SIM_BARNES_HUT;
        nb_sim* core = nullptr;
        int rc = nb_create(&p, &core);
        if (rc) return rc;
        nb_batch* b = new (std::nothrow) nb_batch();
        if (!b) {
            nb_destroy(core);
            return NB_ENOMEM;
        }
        b->base = p;
        b->bh_threshold = bh_threshold;
        b->bh_theta = bh_theta;
        b->core = core;
        if (dev_alloc(&b->next_unit, sizeof(int)) != cudaSuccess || dev_alloc(&b->held, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            nb_batch_destroy(b);
            return NB_ENOMEM;
        }
        *out = b;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_destroy(nb_batch* b) {
    try {
        if (!b) return NB_EINVAL;
        if (b->core) cudaSetDevice(b->core->dev);
        if (b->core && b->core->stream) cudaStreamSynchronize(b->core->stream);
        if (b->exec) cudaGraphExecDestroy(b->exec);
        void* ptrs[] = {b->body_slot, b->gal_range, b->gal_box, b->gal_root, b->slot_start, b->groups, b->group_ctr,
                        b->box_bits, b->cell_rec, b->body_dgal, b->dgal, b->units,
                        b->unit_comp, b->part, b->next_unit, b->held};
        for (void* p : ptrs) dev_free(p, b->core ? b->core->stream : nullptr);
        if (b->core) nb_destroy(b->core);
        delete b;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

const char* nb_batch_last_error(const nb_batch* b) { return b ? b->err.c_str() : "null handle"; }

void* nb_batch_stream(nb_batch* b) { return b && b->core ? (void*)b->core->stream : nullptr; }

int nb_batch_add(nb_batch* b, const float* pos_mass4, const float* vel4, size_t n, int32_t* galaxy) {
    try {
        if (!b || !pos_mass4 || !vel4 || n == 0) return NB_EINVAL;
        if (b->committed) return bfail(b, NB_EBADSTATE, "galaxies are added before nb_batch_commit");
        if (n > kMaxGalaxyBodies) return bfail(b, NB_EINVAL, "galaxy too large for the batched form");
        b->h_pos.emplace_back(pos_mass4, pos_mass4 + 4 * n);
        b->h_vel.emplace_back(vel4, vel4 + 4 * n);
        nb_batch::Gal g;
        g.n = n;
        g.bh = n >= b->bh_threshold;
        b->gal.push_back(g);
        if (galaxy) *galaxy = (int32_t)(b->gal.size() - 1);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_add_generated(nb_batch* b, int model, uint64_t seed, size_t n, int32_t* galaxy) {
    try {
        if (!b || n < 2) return NB_EINVAL;
        if (model < 0 || model > 2) return bfail(b, NB_EINVAL, "unknown galaxy model");
        if (b->committed) return bfail(b, NB_EBADSTATE, "galaxies are added before nb_batch_commit");
        if (n > kMaxGalaxyBodies) return bfail(b, NB_EINVAL, "galaxy too large for the batched form");
        b->h_pos.emplace_back();
        b->h_vel.emplace_back();
        nb_batch::Gal g;
        g.n = n;
        g.bh = n >= b->bh_threshold;
        g.gen_model = model;
        g.gen_seed = seed;
        b->gal.push_back(g);
        if (galaxy) *galaxy = (int32_t)(b->gal.size() - 1);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_steps_not_run(nb_batch* b, int* steps) {
    if (!b || !steps) return NB_EINVAL;
    *steps = b->steps_not_run;
    return NB_OK;
}

int nb_batch_commit(nb_batch* b) {
    try {
        if (!b) return NB_EINVAL;
        if (b->committed) return bfail(b, NB_EBADSTATE, "already committed");
        if (b->gal.empty()) return bfail(b, NB_EINVAL, "no galaxies");
        cudaSetDevice(b->core->dev);
        // layout: Barnes-Hut galaxies packed first (slot order), then direct-sum
        // galaxies padded to multiples of 256 bodies
        size_t off = 0;
        int slot = 0;
        for (auto& g : b->gal)
            if (g.bh) {
                g.off = off;
                g.idx = slot++;
                g.n_pad = g.n;
                off += g.n;
            }
        b->n_bh = off;
        b->nslot = slot;
        if (slot >= (1 << 21)) return bfail(b, NB_EINVAL, "too many Barnes-Hut galaxies");
        off = pad_up(off, 256);
        b->dir_begin = off;
        int dgi = 0;
        for (auto& g : b->gal)
            if (!g.bh) {
                g.off = off;
                g.idx = dgi++;
                g.n_pad = pad_up(g.n, 256);
                off += g.n_pad;
                b->direct_pairs += (uint64_t)g.n * (uint64_t)(g.n - 1);
            }
        b->ndgal = dgi;
        b->n_total = off;
        if (b->n_total > (size_t)INT32_MAX / 2) return bfail(b, NB_EINVAL, "batch too large");
        // per-body galaxy tables, filled on the device from runs of at most
        // kFillChunk bodies (begin, count, galaxy, table: 0 slot of a Barnes-Hut
        // body, 1 direct-sum galaxy of a direct body, -1 on its padding)
        std::vector<int32_t> slot_start(b->nslot);
        std::vector<int4> gal_range(b->nslot), fill;
        b->n_real = 0;
        // state: zeroed arrays (padding bodies are zero-mass at the origin), host
        // galaxies copied in and validated
        int rc = sim_reserve_zeroed(b->core, b->n_total);
        if (rc) return bfail(b, rc, nb_last_error(b->core));
        std::vector<GenSpec> gen;
        for (size_t k = 0; k < b->gal.size(); ++k) {
            const auto& g = b->gal[k];
            if (g.gen_model >= 0) {
                gen.push_back(GenSpec{g.gen_seed, g.off, g.n, g.gen_model});
            } else if (!g.dsrc[0]) {
                NB_BCUDA(b, cudaMemcpyAsync(b->core->pos + g.off, b->h_pos[k].data(), 16 * g.n, cudaMemcpyHostToDevice,
                                            b->core->stream));
                NB_BCUDA(b, cudaMemcpyAsync(b->core->vel + g.off, b->h_vel[k].data(), 16 * g.n, cudaMemcpyHostToDevice,
                                            b->core->stream));
            }
            b->n_real += g.n;
            const size_t t0 = g.bh ? g.off : g.off - b->dir_begin;
            for (size_t c = 0; c < g.n; c += kFillChunk)
                fill.push_back(make_int4((int)(t0 + c), (int)std::min<size_t>(kFillChunk, g.n - c), g.idx, g.bh ? 0 : 1));
            if (g.bh) {
                slot_start[g.idx] = (int)g.off;
                gal_range[g.idx] = make_int4((int)g.off, (int)g.n, 0, 0);
            }
        }
        // galaxies generated on the device, straight into the state arrays
        NB_BCUDA(b, gen_galaxies(gen, b->core->pos, b->core->vel, b->core->stream));
        rc = sim_check_state(b->core);
        if (rc) return bfail(b, rc, nb_last_error(b->core));
        if (b->nslot > 0) {
            // Cell quadrupoles are float sums of m (3 y y - |y|^2): bounded by
            // 12 M x^2 with M the largest member's mass and x the largest
            // coordinate.  States beyond float range (the reference's SI-like
            // masses, 1e20..1e30, at positions of order 1e3) belong to the plain path.
            unsigned h[2] = {0u, 0u};
            NB_BCUDA(b, cudaMemcpy(h, b->core->d_mmax, sizeof(h), cudaMemcpyDeviceToHost));
            float mf, xf;
            std::memcpy(&mf, &h[0], 4);
            std::memcpy(&xf, &h[1], 4);
            size_t nmax = 0;
            for (const auto& g : b->gal)
                if (g.bh) nmax = std::max(nmax, g.n);
            if (12.0 * (double)nmax * (double)mf * (double)xf * (double)xf > 1e37)
                return bfail(b, NB_ENOTSUP, "Barnes-Hut member beyond the float range of the batched form's cell "
                                            "quadrupoles (mass x size^2); use N-body units or the plain path");
        }
        // galaxies handed over from another batch keep their exact state,
        // compensation and last accelerations included
        for (const auto& g : b->gal) {
            if (!g.dsrc[0]) continue;
            float4* dst[5] = {b->core->pos, b->core->posc, b->core->vel, b->core->velc, b->core->acc};
            for (int a = 0; a < 5; ++a)
                NB_BCUDA(b, cudaMemcpyAsync(dst[a] + g.off, g.dsrc[a], g.n * sizeof(float4), cudaMemcpyDeviceToDevice,
                                            b->core->stream));
        }
        NB_BCUDA(b, upload(&b->slot_start, slot_start, b->core->stream));
        NB_BCUDA(b, upload(&b->gal_range, gal_range, b->core->stream));
        {
            cudaStream_t st = b->core->stream;
            dev_free(b->body_slot, st);
            dev_free(b->body_dgal, st);
            b->body_slot = b->body_dgal = nullptr;
            if (b->n_bh > 0) NB_BCUDA(b, dev_alloc(&b->body_slot, b->n_bh * sizeof(int32_t)));
            const size_t nd = b->n_total - b->dir_begin;
            if (nd > 0) {
                NB_BCUDA(b, dev_alloc(&b->body_dgal, nd * sizeof(int32_t)));
                NB_BCUDA(b, cudaMemsetAsync(b->body_dgal, 0xff, nd * sizeof(int32_t), st));   // padding: -1
            }
            int4* d_fill = nullptr;
            NB_BCUDA(b, upload(&d_fill, fill, st));
            if (!fill.empty())
                k_fill_tables<<<(unsigned)fill.size(), 256, 0, st>>>(d_fill, b->body_slot, b->body_dgal);
            const cudaError_t e = cudaGetLastError();
            dev_free(d_fill, st);
            NB_BCUDA(b, e);
        }
        if (b->nslot > 0) {
            NB_BCUDA(b, dev_alloc(&b->gal_box, b->nslot * sizeof(float4)));
            NB_BCUDA(b, dev_alloc(&b->gal_root, b->nslot * sizeof(int32_t)));
            NB_BCUDA(b, dev_alloc(&b->box_bits, 6 * b->nslot * sizeof(unsigned)));
            // groups are disjoint and non-empty: at most one per body
            b->group_cap = (int)b->n_bh;
            NB_BCUDA(b, dev_alloc(&b->groups, b->n_bh * sizeof(int4)));
            NB_BCUDA(b, dev_alloc(&b->group_ctr, 2 * sizeof(int)));
        }
        b->h_pos.clear();
        b->h_vel.clear();
        rc = plan_units(b);
        if (rc) return rc;
        rc = size_tree(b);
        if (rc) return rc;
        b->committed = true;
        return sync_check(b);
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_set_tuning(nb_batch* b, const nb_tuning* t) {
    try {
        if (!b || !t) return NB_EINVAL;
        if (!tuning_valid(*t)) return bfail(b, NB_EINVAL, "unsupported tuning");
        b->tune = *t;
        b->graph_dirty = true;
        if (!b->committed) return NB_OK;
        cudaSetDevice(b->core->dev);
        return plan_units(b);
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_set_far_accuracy(nb_batch* b, double alpha, double eta_max) {
    try {
        if (!b) return NB_EINVAL;
        if (!(alpha >= 0.0) || !(eta_max > 0.0) || eta_max >= 1.0)
            return bfail(b, NB_EINVAL, "far-field alpha must be >= 0 and eta_max in (0, 1)");
        b->far_alpha = alpha;
        b->far_cap = eta_max;
        b->graph_dirty = true;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_set_far_field(nb_batch* b, double eta) {
    try {
        if (!b) return NB_EINVAL;
        if (!(eta >= 0.0) || eta >= 1.0) return bfail(b, NB_EINVAL, "far-field eta must be in [0, 1)");
        b->far_eta = eta;
        b->graph_dirty = true;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_get_tuning(nb_batch* b, nb_tuning* t) {
    try {
        if (!b || !t) return NB_EINVAL;
        *t = b->tune;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_step(nb_batch* b, float dt, int nsteps) {
    try {
        const int rc = nb::batch_launch_steps(b, dt, nsteps);
        return rc ? rc : nb::batch_wait(b);
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_read(nb_batch* b, int32_t galaxy, float* pos_mass4, float* vel4) {
    try {
        if (!b) return NB_EINVAL;
        const nb_batch::Gal* g = find(b, galaxy);
        if (!g || !b->committed) return bfail(b, NB_EINVAL, "unknown galaxy or not committed");
        cudaSetDevice(b->core->dev);
        nb_sim* c = b->core;
        const size_t n = g->n;
        std::vector<float4> v(n), vc(n);
        if (pos_mass4) NB_BCUDA(b, cudaMemcpy(pos_mass4, c->pos + g->off, n * 16, cudaMemcpyDeviceToHost));
        if (vel4) {
            NB_BCUDA(b, cudaMemcpy(v.data(), c->vel + g->off, n * 16, cudaMemcpyDeviceToHost));
            NB_BCUDA(b, cudaMemcpy(vc.data(), c->velc + g->off, n * 16, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < n; ++i) {
                vel4[4 * i] = (float)((double)v[i].x - vc[i].x);
                vel4[4 * i + 1] = (float)((double)v[i].y - vc[i].y);
                vel4[4 * i + 2] = (float)((double)v[i].z - vc[i].z);
                vel4[4 * i + 3] = 0.f;
            }
        }
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_forces(nb_batch* b, int32_t galaxy, double* force3) {
    try {
        if (!b || !force3) return NB_EINVAL;
        const nb_batch::Gal* g = find(b, galaxy);
        if (!g || !b->committed) return bfail(b, NB_EINVAL, "unknown galaxy or not committed");
        cudaSetDevice(b->core->dev);
        int rc = enqueue_step(b, 0.f, false);
        if (rc) return rc;
        bool fits = true;
        rc = sync_check(b, &fits);
        if (rc) return rc;
        if (!fits) {   // the tree outgrew its arrays: size it from this state and evaluate again
            rc = size_tree(b);
            if (!rc) rc = enqueue_step(b, 0.f, false);
            if (!rc) rc = sync_check(b);
            if (rc) return rc;
        }
        nb_sim* c = b->core;
        std::vector<float4> a(g->n), p(g->n);
        NB_BCUDA(b, cudaMemcpy(a.data(), c->acc + g->off, g->n * 16, cudaMemcpyDeviceToHost));
        NB_BCUDA(b, cudaMemcpy(p.data(), c->pos + g->off, g->n * 16, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < g->n; ++i) {
            const double m = p[i].w;
            force3[3 * i] = m * a[i].x;
            force3[3 * i + 1] = m * a[i].y;
            force3[3 * i + 2] = m * a[i].z;
        }
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_launch_count(nb_batch* b, uint64_t* launches) {
    try {
        if (!b || !launches) return NB_EINVAL;
        *launches = b->core ? b->core->prof.launches : 0;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_info(nb_batch* b, size_t* galaxies, size_t* bodies, uint64_t* interactions_last) {
    try {
        if (!b) return NB_EINVAL;
        if (galaxies) *galaxies = b->gal.size();
        if (bodies) *bodies = b->committed ? b->n_real : 0;
        if (interactions_last) {
            unsigned long long v = 0;
            if (b->committed && b->n_bh > 0) {
                cudaSetDevice(b->core->dev);
                NB_BCUDA(b, cudaMemcpy(&v, b->core->tree.interactions, sizeof(v), cudaMemcpyDeviceToHost));
            }
            *interactions_last = (uint64_t)v + b->direct_pairs;
        }
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_batch_tree_stats(nb_batch* b, int64_t* stats4) {
    try {
        if (!b || !stats4) return NB_EINVAL;
        for (int k = 0; k < 4; ++k) stats4[k] = 0;
        if (!b->committed || b->n_bh == 0) return NB_OK;
        cudaSetDevice(b->core->dev);
        int32_t h[TC_COUNT];
        int rc = read_tree_counts(b, h);
        if (rc) return rc;
        int ctr[2] = {0, 0};
        NB_BCUDA(b, cudaMemcpy(ctr, b->group_ctr, sizeof(ctr), cudaMemcpyDeviceToHost));
        stats4[0] = ctr[0];
        stats4[1] = h[TC_NINT];
        stats4[2] = (int64_t)h[TC_NINT] + h[TC_NLEAF];
        stats4[3] = (int64_t)b->n_bh;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

// Project autotuner: candidate leaf sizes for the Barnes-Hut members, then
// candidate direct-sum tilings, each timed over trial_steps graph replays with
// CUDA events; the state is restored after every trial.
int nb_batch_autotune(nb_batch* b, float dt, int trial_steps) {
    try {
        if (!b) return NB_EINVAL;
        if (!b->committed) return bfail(b, NB_EBADSTATE, "nb_batch_commit first");
        if (trial_steps < 1) return bfail(b, NB_EINVAL, "trial_steps >= 1");
        cudaSetDevice(b->core->dev);
        // the trials step from the current state: size the tree for it (a state
        // written since the commit may need more nodes)
        int rc = size_tree(b);
        if (rc) return rc;
        nb_sim* c = b->core;
        const size_t bytes = c->n_pad * sizeof(float4);
        float4* save = nullptr;
        NB_BCUDA(b, dev_alloc(&save, 5 * bytes));
        // the state and the accelerations the far field's relative rule reads
        auto snapshot = [&](bool restore) {
            float4* arrs[5] = {c->pos, c->posc, c->vel, c->velc, c->acc};
            for (int k = 0; k < 5; ++k) {
                if (restore) cudaMemcpyAsync(arrs[k], save + k * c->n_pad, bytes, cudaMemcpyDeviceToDevice, c->stream);
                else cudaMemcpyAsync(save + k * c->n_pad, arrs[k], bytes, cudaMemcpyDeviceToDevice, c->stream);
            }
        };
        snapshot(false);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        auto trial = [&](const nb_tuning& t, float* ms) -> int {
            int rc = nb_batch_set_tuning(b, &t);
            if (rc) return rc;
            rc = build_graph(b, dt);
            if (rc) return rc;
            cudaGraphLaunch(b->exec, c->stream);   // warm-up
            cudaEventRecord(e0, c->stream);
            for (int k = 0; k < trial_steps; ++k) cudaGraphLaunch(b->exec, c->stream);
            cudaEventRecord(e1, c->stream);
            rc = sync_check(b);
            if (rc) return rc;
            cudaEventElapsedTime(ms, e0, e1);
            snapshot(true);
            return NB_OK;
        };
        nb_tuning best = b->tune;
        float best_ms = INFINITY;
        const int leafs[] = {8, 16, 32, 64};
        for (int ls : (b->n_bh > 0 ? std::vector<int>(leafs, leafs + 4) : std::vector<int>{best.leaf_size})) {
            nb_tuning t = best;
            t.leaf_size = ls;
            float ms = 0.f;
            rc = trial(t, &ms);
            if (rc) break;
            if (ms < best_ms) { best_ms = ms; best = t; }
        }
        const int shapes[][3] = {{128, 1, 1024}, {128, 2, 1024}, {64, 1, 1024}, {128, 1, 2048}, {256, 1, 1024}, {128, 2, 2048}};
        if (!rc && b->ndgal > 0) {
            const nb_tuning base_t = best;
            for (const auto& sh : shapes) {
                nb_tuning t = base_t;
                t.direct_block = sh[0];
                t.direct_ipt = sh[1];
                t.direct_jtile = sh[2];
                float ms = 0.f;
                rc = trial(t, &ms);
                if (rc) break;
                if (ms < best_ms) { best_ms = ms; best = t; }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        snapshot(true);
        cudaStreamSynchronize(c->stream);
        dev_free(save, c->stream);
        if (rc) return rc;
        return nb_batch_set_tuning(b, &best);
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

}  // extern "C"

// ---- whole-batch state transfer (the reference-facing end-to-end path) -----
extern "C" {

// Uploads the state of every galaxy (galaxies in index order, concatenated:
// n_bodies x float4 each) from host buffers; the tree and graph are reused.
int nb_batch_write_state(nb_batch* b, const float* pos_mass4, const float* vel4) {
    try {
        if (!b || !pos_mass4 || !vel4) return NB_EINVAL;
        if (!b->committed) return bfail(b, NB_EBADSTATE, "nb_batch_commit first");
        cudaSetDevice(b->core->dev);
        nb_sim* c = b->core;
        size_t src = 0;
        for (const auto& g : b->gal) {
            NB_BCUDA(b, cudaMemcpyAsync(c->pos + g.off, pos_mass4 + 4 * src, g.n * 16, cudaMemcpyHostToDevice, c->stream));
            NB_BCUDA(b, cudaMemcpyAsync(c->vel + g.off, vel4 + 4 * src, g.n * 16, cudaMemcpyHostToDevice, c->stream));
            NB_BCUDA(b, cudaMemsetAsync(c->posc + g.off, 0, g.n * 16, c->stream));
            NB_BCUDA(b, cudaMemsetAsync(c->velc + g.off, 0, g.n * 16, c->stream));
            src += g.n;
        }
        // accelerations belong to the previous state: the next evaluation takes
        // the far field's geometric rule, as after a commit
        NB_BCUDA(b, cudaMemsetAsync(c->acc, 0, c->n_pad * sizeof(float4), c->stream));
        // validated (reported by the next wait) and the largest mass recorded
        const int rc = sim_rescan_state(c);
        if (rc) return bfail(b, rc, nb_last_error(c));
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

// Downloads positions+masses (and, if vel4 is not NULL, velocities) of every
// galaxy into host buffers in the same concatenated order.
int nb_batch_read_state(nb_batch* b, float* pos_mass4, float* vel4) {
    try {
        if (!b || !pos_mass4) return NB_EINVAL;
        if (!b->committed) return bfail(b, NB_EBADSTATE, "nb_batch_commit first");
        cudaSetDevice(b->core->dev);
        nb_sim* c = b->core;
        size_t dst = 0;
        for (const auto& g : b->gal) {
            NB_BCUDA(b, cudaMemcpyAsync(pos_mass4 + 4 * dst, c->pos + g.off, g.n * 16, cudaMemcpyDeviceToHost, c->stream));
            if (vel4)
                NB_BCUDA(b, cudaMemcpyAsync(vel4 + 4 * dst, c->vel + g.off, g.n * 16, cudaMemcpyDeviceToHost, c->stream));
            dst += g.n;
        }
        NB_BCUDA(b, cudaStreamSynchronize(c->stream));
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

}  // extern "C"
