// nb_internal.hpp -- host-side state of a simulator handle and the kernel
// launchers shared between translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include "../../include/nbody_gb300.h"
#include "nb_common.cuh"

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
//
// Bodies are sorted by their octant path (key); the tree keeps every
// non-empty node as a "cell".  Cell 0 is the root; the non-empty children of
// an internal node occupy consecutive cells in octant order.
struct TreeBuffers {
    size_t body_cap = 0;   // sort capacity (multiple of the sort tile)
    size_t int_cap = 0;    // internal nodes
    size_t cell_cap = 0;   // cells
    size_t hash_cap = 0;   // power of two
    // per body
    uint64_t* keys[2] = {nullptr, nullptr};  // radix ping-pong (input order in [0] before the sort)
    int32_t* vals[2] = {nullptr, nullptr};   // original index per sorted position
    int32_t* depth = nullptr;                // levels descended (input order)
    float4* spos = nullptr;                  // positions in sorted order
    int32_t* pos_nint = nullptr;             // internal nodes starting at a position (scanned in place)
    int32_t* leaf_level = nullptr;           // level of the leaf starting at a position, -1 if none
    int32_t* leaf_count = nullptr;           // bodies of that leaf
    int32_t* leaf_parent = nullptr;          // internal node holding that leaf
    // per internal node (numbered by first body, then level)
    int32_t* int_level = nullptr;
    int32_t* int_first = nullptr;
    int32_t* int_parent = nullptr;
    uint32_t* int_mask = nullptr;            // non-empty child octants
    int32_t* int_nint = nullptr;             // internal children
    int32_t* int_pending = nullptr;          // bottom-up arrivals
    int32_t* int_block = nullptr;            // first child cell
    int32_t* int_cell = nullptr;             // own cell
    uint64_t* int_code = nullptr;            // (1 << 3 level) | prefix
    // per cell
    float4* cell_com = nullptr;              // (centre of mass, float(TotalMass))
    int4* cell_meta = nullptr;               // (first child cell | first sorted body, accept r^2, reject r^2,
                                             //  kind | nchild << 4 | bucket count << 8)
    int32_t* cell_count = nullptr;           // NumParticles
    double* cell_mass = nullptr;             // TotalMass
    float4* cell_lo = nullptr;               // (TopLeft.xyz, side)
    float4* cell_hi = nullptr;               // (BottomRight.xyz, level)
    uint64_t* cell_code = nullptr;           // (1 << 3 level) | prefix
    // internal node lookup by code
    uint64_t* hkeys = nullptr;
    int32_t* hvals = nullptr;
    // radix sort and the single-pass scans (decoupled look-back)
    uint32_t* ghist = nullptr;               // [pass][digit], inside the counters buffer
    int32_t* plan = nullptr;                 // [0..7] skip, [8..15] source buffer, [16] final buffer
    int32_t* dig_off = nullptr;              // [pass][digit]: where the digit's keys start
    unsigned long long* sort_status = nullptr;   // [pass][tile][digit]
    unsigned long long* pos_status = nullptr;    // [tile]: positions scan (body_cap / sort tile)
    unsigned long long* popc_status = nullptr;   // [tile]: child-count scan (int_cap / sort tile)
    // counters (device: kCounterWords words, then ghist) and their pinned host mirror
    int32_t* counters = nullptr;
    int32_t* h_counters = nullptr;
    unsigned long long* interactions = nullptr;
    // host view of the last build
    int n_in = 0, n_int = 0, n_cells = 0, final_buf = 0;
    bool trivial = false;                    // < 2 bodies in the tree: all forces zero
};

// Tree counters (TreeBuffers::counters)
enum : int {
    TC_NIN = 0,       // bodies inside the root cube
    TC_NINT = 1,      // internal nodes
    TC_NLEAF = 2,     // leaf cells
    TC_GAPS = 3,      // bodies whose path met a gap between float child bounds
    TC_DEEPER = 4,    // depth-cap buckets whose bodies differ (the reference would split further)
    TC_HASHFAIL = 5,  // failed internal-node lookups (must stay 0)
    TC_OVERFLOW = 6,  // nodes beyond the allocated capacity (must stay 0)
    TC_COUNT = 8,     // the counters above are read by the host
    // tile counters of the look-back kernels (blocks take tiles in start order)
    TC_TILE_POS = 8,
    TC_TILE_POPC = 9,
    TC_TILE_SORT = 10,   // one per radix pass
};
constexpr int kCounterWords = 32;   // counters before the radix histograms in the same buffer

#ifdef __CUDACC__
// Whether a tree built over fixed capacities (int_cap internal nodes,
// cell_cap cells) without a host check of its counts fits them.  The counts
// are final once the topology kernels have run.
__device__ __forceinline__ bool tree_fits(const int32_t* counters, int int_cap, int cell_cap) {
    const int ni = counters[TC_NINT];
    return (counters[TC_OVERFLOW] | counters[TC_HASHFAIL]) == 0 && ni <= int_cap &&
           ni + counters[TC_NLEAF] <= cell_cap;
}
#endif

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
    int pageable_access = 0;   // cudaDevAttrPageableMemoryAccess: kernels may address the caller's host records
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
    // render hand-off: when attached, every kick-drift also writes the vertex
    // (position, colour, scale) of each body it moves
    nb_render_vertex* render = nullptr;
    float4* rcolour = nullptr;
    float rscale = 1.f;
    // staging of the record boundary (nb_init_particles, nb_write_back,
    // nb_read_state): grown on demand and kept, so that a step through the
    // C-ABI allocates nothing
    void* d_stage = nullptr;
    size_t d_stage_bytes = 0;
    void* h_stage = nullptr;   // pinned
    size_t h_stage_bytes = 0;
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
    // float bits of the state's largest |mass| (the direct sum's self-pair
    // guard) and of its largest |coordinate|, recorded when a state is loaded
    unsigned* d_mmax = nullptr;
    // the largest mass as last read back: above 1e21 the direct-sum force
    // kernel takes its self-pair guard from d_mmax (its heavy variant)
    bool heavy = false;
    int* h_err = nullptr;     // pinned: [0] mirror of d_err, [1] init's non-zero-force flag, [2..3] of d_mmax
    unsigned long long* d_inter = nullptr;
    uint64_t inter_last = 0;
    bool forces_fresh = false;  // acc holds the forces of the current positions
    nb::Profiler prof{};
    bool tune_set = false;     // direct-sum tuning set through nb_tune (else sized by n)
    // polls of each source-tile wait of the direct-sum force kernel before the
    // step is abandoned (nb_tune "wait_polls"; lowered only by the test of the
    // timeout path)
    uint32_t wait_polls = nb::kMaxPolls;
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
// hold (device tree counters, optional): a step whose tree does not fit
// int_cap / cell_cap leaves the state unchanged and adds one to *held.
cudaError_t kick_drift(nb_sim* sim, float dt, const int32_t* hold = nullptr, int int_cap = 0, int cell_cap = 0,
                       int* held = nullptr);

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
float theta_float(double theta);   // smallest float >= theta
// Batched form: topology of pre-computed keys without host synchronisation.
// counts_only: stop once the node counts are known (no node is written, so
// the node arrays may still be too small for the tree).  rec: the batched
// form's cell records; its leaves are placed there (nb_cellrec.cuh) instead of
// the plain path's per-cell arrays, and internal nodes get only their cell.
struct CellRec;
cudaError_t tree_build_graph(nb_sim* sim, const float4* pos, int n, int D, bool counts_only = false,
                             CellRec* rec = nullptr);
// Words of the counters buffer (counters, tile counters, radix histograms)
// that a batched step clears before its keys.
int tree_counter_words();
// Keys of the batched forest with the sort's histograms; writes each
// galaxy's cube (x0, y0, z0, edge) from its ordered min/max words.
cudaError_t tree_batch_keys(nb_sim* sim, const float4* pos, const int32_t* body_slot, int n,
                            const unsigned* box_bits, int nslot, float4* gal_box);
cudaError_t tree_reserve_graph(nb_sim* sim, int n, size_t n_int, size_t n_cells);
int tree_sort_tile();

// ---- state set-up without a host copy of every body (nb_api.cu) ----
// Sizes the state arrays for n bodies, all zero (zero-mass bodies at the
// origin), for the caller to fill by copies on sim->stream.
int sim_reserve_zeroed(nb_sim* s, size_t n);
// Validates positions and velocities (finite) and zeroes the compensation
// arrays, as nb_init_soa does after its upload; records the largest mass.
int sim_check_state(nb_sim* s);
// The same without waiting: a non-finite value is reported by the next
// synchronisation.
int sim_rescan_state(nb_sim* s);

// ---- batched form hand-over (nb_batch.cu), used by the served form ----
constexpr size_t kMaxGalaxyBodies = (size_t)1 << 24;   // bodies of one galaxy in the batched form
// A galaxy handed over keeps its state, its compensation terms and its last
// accelerations (the relative far-field rule of the next step reads them).
int batch_add_device(nb_batch* b, const float4* pos, const float4* posc, const float4* vel, const float4* velc,
                     const float4* acc, size_t n, int32_t* galaxy);
int batch_device_state(nb_batch* b, int32_t galaxy, const float4** pos, const float4** posc, const float4** vel,
                       const float4** velc, const float4** acc, size_t* n);
// nb_batch_step in two halves: enqueue the steps, then wait for them and check
// the device's error and overflow flags.
int batch_launch_steps(nb_batch* b, float dt, int nsteps);
int batch_wait(nb_batch* b);
// Steps of the last launch that were not run when batch_wait failed with
// NB_ENOMEM (the octree kept outgrowing its arrays); 0 otherwise.
int batch_steps_not_run(const nb_batch* b);

// ---- galaxies generated on the device (nb_gen.cu) ----
// model: 0 exponential disk + 10% Hernquist bulge, 1 Plummer sphere, 2 two
// Plummer spheres on a parabolic orbit (the host generators' defaults).
struct GenSpec {
    uint64_t seed;
    size_t off;   // first body in the state arrays
    size_t n;
    int model;
};
cudaError_t gen_galaxies(const std::vector<GenSpec>& specs, float4* pos, float4* vel, cudaStream_t st);

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

// ---- device memory (nb_api.cu) ----
// The library's device buffers come from one memory pool per device that
// keeps freed memory for later allocations: a served batch rebuilt every few
// rounds allocates and frees gigabytes, which cudaMalloc / cudaFree would map
// and unmap each time (and every cudaFree waits for the whole device).
// dev_alloc: the buffer may be used on any stream when it returns.
// dev_free: returns the buffer after the work already queued on st (the
// stream every use of the buffer was queued on).
cudaError_t dev_alloc(void** p, size_t bytes);
template <typename T>
cudaError_t dev_alloc(T** p, size_t bytes) {
    return dev_alloc(reinterpret_cast<void**>(p), bytes);
}
void dev_free(void* p, cudaStream_t st);

// ---- misc ----
cudaError_t render_fill(nb_sim* sim, const float4* d_colour, float scale, nb_render_vertex* d_out);

}  // namespace nb
