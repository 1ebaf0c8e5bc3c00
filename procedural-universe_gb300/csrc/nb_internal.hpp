// nb_internal.hpp -- host-side state of a simulator handle and the kernel
// launchers shared between translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include "../../include/nbody_gb300.h"

namespace nb {

// Padding of the body arrays: every array holds a multiple of kPad entries;
// padded entries are zero-mass bodies at the origin, which contribute exactly
// zero force, so kernels never need a ragged tail.
constexpr int kPad = 2048;
constexpr int kTileJ = 128;   // source bodies per shared-memory tile

inline size_t pad_up(size_t n, size_t m) { return (n + m - 1) / m * m; }

// Tuning of the direct-sum kernel.
struct DirectTuning {
    int block = 128;   // threads per block
    int ipt = 4;       // target bodies per thread
    int splits = 0;    // source ranges per target block (0 = automatic)
};

// Device arrays of a Barnes-Hut octree (structure of arrays).
struct TreeBuffers {
    size_t node_cap = 0;        // capacity in cells
    size_t body_cap = 0;
    // per body (sorted order and keys)
    uint64_t* keys = nullptr;      // octant path (63 bits) per body, input order
    uint64_t* keys_alt = nullptr;  // radix sort ping-pong
    int32_t* order = nullptr;      // body index at each sorted position
    int32_t* order_alt = nullptr;
    int32_t* depth = nullptr;      // levels descended per body (input order)
    uint8_t* delta = nullptr;      // common levels of sorted neighbours i, i+1
    int32_t* own_scan = nullptr;   // per sorted position: internal nodes it opens (scanned)
    int32_t* close_pos = nullptr;  // scratch for range ends
    // per cell (internal + leaf cells), cell 0 = root
    float4* cell_com = nullptr;    // (com.x, com.y, com.z, float(mass))
    double* cell_mass = nullptr;   // TotalMass
    int32_t* cell_child = nullptr; // internal: first child cell; leaf: -1
    int32_t* cell_count = nullptr; // bodies in the subtree
    int32_t* cell_first = nullptr; // first sorted position of the subtree
    float4* cell_lo = nullptr;     // (TopLeft.xyz, side)
    int32_t* cell_level = nullptr;
    uint64_t* cell_prefix = nullptr;
    int32_t* cell_parent = nullptr;
    int32_t* cell_pending = nullptr;  // bottom-up arrival counters
    int32_t* counters = nullptr;      // [0] cells used, [1] internal nodes, [2] max level, ...
    // radix sort scratch
    uint32_t* hist = nullptr;      // per-block digit histograms
    size_t hist_cap = 0;
    int32_t* sort_state = nullptr; // device-side pass control
    // traversal output
    unsigned long long* interactions = nullptr;
};

// Phases timed by the per-handle profiler (NB_PHASE_* in the public header).
constexpr int kPhases = 10;

// CUDA-event timing of kernel phases on the handle's stream.
struct Profiler {
    bool on = false;
    struct Pending {
        int phase;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    double ms[kPhases] = {};
    uint64_t count[kPhases] = {};
    uint64_t launches = 0;   // kernel launches issued by this handle (profiled or not)
};

}  // namespace nb

struct nb_sim {
    nb_params prm{};
    int dev = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    size_t n = 0;        // bodies
    size_t n_pad = 0;    // padded count
    size_t cap = 0;      // allocated padded capacity
    // state (device)
    float4* pos = nullptr;    // x, y, z, m
    float4* posc = nullptr;   // Kahan compensation of the position
    float4* vel = nullptr;    // vx, vy, vz, 0
    float4* velc = nullptr;   // Kahan compensation of the velocity
    float4* acc = nullptr;    // acceleration of the last force evaluation (G applied)
    float4* finit = nullptr;  // initial forces / m from the records, applied once (direct sum)
    bool finit_pending = false;
    // direct-sum partial sums
    float4* part = nullptr;   // [splits][n_pad] sums then [splits][n_pad] compensations
    size_t part_cap = 0;      // in float4 entries
    nb::DirectTuning tune{};
    // Barnes-Hut
    nb::TreeBuffers tree{};
    bool tree_valid = false;
    // diagnostics scratch
    double* dscratch = nullptr;
    size_t dscratch_cap = 0;
    int* d_err = nullptr;     // device error word
    int* h_err = nullptr;     // pinned mirror
    unsigned long long* d_inter = nullptr;
    uint64_t inter_last = 0;
    bool forces_fresh = false;  // acc holds the forces of the current positions
    nb::Profiler prof{};
    std::string err;
};

namespace nb {

// ---- direct sum (nb_direct.cu) ----
// Launches the force kernel for all bodies of `sim` and reduces the partials
// into sim->acc (G applied, initial forces added when pending). When dt != 0
// the same reduction kernel also performs the kick-drift update.
cudaError_t direct_force_update(nb_sim* sim, float dt, bool update);
int direct_splits(const nb_sim* sim, const DirectTuning& t, size_t n_pad);
size_t direct_part_entries(const nb_sim* sim, const DirectTuning& t, size_t n_pad);

// Generic kick-drift of bodies from sim->acc (used after a Barnes-Hut force pass).
cudaError_t kick_drift(nb_sim* sim, float dt);

// ---- FP64 oracle and diagnostics (nb_fp64.cu) ----
cudaError_t fp64_forces(nb_sim* sim, const int32_t* d_targets, size_t m, double* d_out3);
cudaError_t fp64_diagnostics(nb_sim* sim, double* d_out /* 12 doubles */);
cudaError_t fp64_diagnostics_ex(nb_sim* sim, float half_dt, bool with_acc, bool with_potential, double* d_out);

// ---- Barnes-Hut (nb_tree.cu, nb_traverse.cu) ----
cudaError_t tree_reserve(nb_sim* sim);
void tree_free(nb_sim* sim);
cudaError_t tree_build(nb_sim* sim);
cudaError_t tree_forces(nb_sim* sim);
cudaError_t tree_sizes(nb_sim* sim, int32_t* cells, int32_t* internal);

// ---- profiling (nb_api.cu) ----
// Records CUDA events around one phase on sim->stream when profiling is on
// and counts `launches` kernel launches in either case.
class PhaseScope {
  public:
    PhaseScope(nb_sim* sim, int phase, int launches = 1);
    ~PhaseScope();
  private:
    nb_sim* sim_;
    int phase_;
    cudaEvent_t b_ = nullptr;
};

// ---- misc ----
cudaError_t render_fill(nb_sim* sim, const float4* d_colour, float scale, nb_render_vertex* d_out);

}  // namespace nb
