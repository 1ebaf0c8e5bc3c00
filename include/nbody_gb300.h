/*
 * nbody_gb300.h -- C-ABI of the GB300 N-body step.
 *
 * This is the drop-in boundary for the simulator interface of
 * Procedural-Universe (src/Sim/INBodySim.hpp:19-25):
 *
 *     class INBodySim {
 *         virtual void Init(std::vector<Particle>& particles) = 0;
 *         virtual void Update(float dt) = 0;
 *         virtual void RenderDebug(Matrix view, Matrix proj) {}
 *     };
 *     std::unique_ptr<INBodySim> CreateNBodySim(ID3D11DeviceContext*, ENBodySim);
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (NB_OK or a negative NB_E* code). No C++ exception crosses the boundary.
 * A handle's calls must be serialised by the caller (the reference calls its
 * simulator from one thread only); different handles may be used from
 * different threads.  All compute runs as CUDA kernels on one GPU; there is
 * no CPU fallback: on a machine without a usable GPU nb_create fails with
 * NB_ECUDA.
 *
 * include/cuda_nbody_sim.hpp wraps these calls in a C++ class with the
 * reference's Init/Update shape.
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NB_OK         0
#define NB_EINVAL    -1   /* bad argument (null pointer, size, NaN/inf input, bad params) */
#define NB_ENOMEM    -2   /* device or host allocation failed / over the memory budget   */
#define NB_ECUDA     -3   /* a CUDA runtime call failed (message in nb_last_error)      */
#define NB_ETIMEOUT  -4   /* a bounded device-side wait ran out; the step was abandoned */
#define NB_EBADSTATE -5   /* call out of order (e.g. nb_step before nb_init_*)           */
#define NB_ENOTSUP   -6   /* combination of options not supported                        */

/* ---- simulator kinds: mirrors ENBodySim (src/Sim/INBodySim.hpp:11-17) ---- */
#define NB_SIM_BRUTE_FORCE   0   /* BruteForceCPU (src/Sim/BruteForceCPU.cpp)            */
#define NB_SIM_BRUTE_FORCE_GPU 1 /* BruteForceGPU: same direct sum, same kernels as 0    */
#define NB_SIM_BARNES_HUT    2   /* BarnesHut + Octree (src/Sim/BarnesHut.cpp, Octree.cpp) */

/* ---- force laws ---------------------------------------------------------- */
/* Reference law, Phys::Gravity (src/Sim/Physics.hpp:25-35):
 *     F_i = sum_j -G m_i m_j / (|p_i-p_j|^2 + S) * normalize(p_i - p_j)
 * with S = softening2.  Plummer law: F_i = sum_j G m_i m_j (p_j-p_i) / (r^2+S)^{3/2}. */
#define NB_LAW_REFERENCE 0
#define NB_LAW_PLUMMER   1

/* Reference record, struct Particle (src/Render/Misc/Particle.hpp:8-18):
 * 104 bytes, Position float3 @0, Colour float4 @12, OriginalColour float4 @28,
 * 4 bytes padding @44, Velocity double3 @48, Forces double3 @72, Mass double @96.
 * This is also the record of the .nbody file format. */
typedef struct nb_particle {
    float  position[3];
    float  colour[4];
    float  original_colour[4];
    float  _pad;
    double velocity[3];
    double forces[3];
    double mass;
} nb_particle;

/* Light-weight render record, LWParticle (src/Render/Misc/Particle.hpp:20-25). */
typedef struct nb_render_vertex {
    float position[3];
    float colour[4];
    float scale;
} nb_render_vertex;

/* Parameters. Fields default (nb_default_params) to the values of the
 * reference configuration translated to N-body units:
 *   G          Phys::G            (src/Sim/Physics.hpp:9)      default 1
 *   softening2 Phys::S            (src/Sim/Physics.hpp:10)     default 1e-4 (eps = 0.01)
 *   theta      Octree::Theta      (src/Sim/Octree.cpp:5)       default 0.5
 *   pos_scale  Phys::StarSystemScale divisor of the drift (src/Sim/BruteForceCPU.cpp:66) default 1
 *   bounds_half half-width of the Barnes-Hut root cube (src/Sim/BarnesHut.cpp:14-21) default 4000
 *   max_depth  octree depth cap (the reference has none; 21 = 63-bit keys)
 *   leaf_size  bodies per leaf before a split (reference: 1)                                */
typedef struct nb_params {
    int    kind;          /* NB_SIM_* */
    int    law;           /* NB_LAW_* */
    double G;
    double softening2;
    double theta;
    double pos_scale;
    float  bounds_half;
    int    max_depth;     /* 1..21 */
    int    leaf_size;     /* >= 1 */
    int    device;        /* CUDA device ordinal */
    void*  stream;        /* cudaStream_t to launch on, or NULL for a library-owned stream */
    int    flags;         /* NB_FLAG_* */
} nb_params;

#define NB_FLAG_NONE            0
#define NB_FLAG_NO_COMPENSATION 1  /* plain FP32 accumulation and update (for error studies) */
/* Where the GPU can address pageable host memory (Grace-attached GPUs report
 * cudaDevAttrPageableMemoryAccess), nb_write_back rewrites the caller's
 * records directly from a kernel instead of copying to a staging buffer and
 * scattering on the host; this flag forces the staged path (same results). */
#define NB_FLAG_STAGED_IO 2

/* FP64 diagnostics: energy, linear momentum, angular momentum (all FP64
 * reductions on the GPU). The potential is the one of the selected law:
 * reference law phi(r) = -(G mi mj / eps)(pi/2 - atan(r/eps)); Plummer
 * phi(r) = -G mi mj / sqrt(r^2 + eps^2). */
typedef struct nb_diag {
    double kinetic;
    double potential;
    double total;
    double momentum[3];
    double angular_momentum[3];
    double mass;
    double centre_of_mass[3];
} nb_diag;

typedef struct nb_sim nb_sim;

int  nb_default_params(nb_params* params);

/* CreateNBodySim (src/Sim/INBodySim.cpp:7-27). */
int  nb_create(const nb_params* params, nb_sim** out);
int  nb_destroy(nb_sim* sim);
const char* nb_last_error(const nb_sim* sim);   /* message of the last failed call, "" if none */
const char* nb_sim_name(int kind);              /* NBodySimGetName (src/Sim/INBodySim.cpp:29-39) */

/* INBodySim::Init (src/Sim/BruteForceCPU.cpp:20-23, src/Sim/BarnesHut.cpp:39-42,
 * src/Sim/BruteForceGPU.cpp:38-43): uploads n reference records. Masses are
 * rounded to float on the device (exact for float-representable masses, which
 * every seeder in this library produces). May be called again with another n. */
int  nb_init_particles(nb_sim* sim, const nb_particle* particles, size_t n);
/* Same from structure-of-arrays host buffers: pos_mass = n x (x,y,z,m),
 * vel = n x (vx,vy,vz,unused). */
int  nb_init_soa(nb_sim* sim, const float* pos_mass4, const float* vel4, size_t n);
/* A reference seeder run on the GPU, then Init: the seeder's
 * Seed(particles) followed by Init(particles) (src/Sim/IParticleSeeder.hpp:12-50,
 * src/States/Simulation/SimulationState.cpp:167-171) without host records.
 * seeder 0 = RandomSeeder, 1 = GalaxySeeder, 2 = StarSystemSeeder (same
 * distributions and bodies as nb_seed_reference); records_out (n records,
 * may be null) receives the generated records. */
int  nb_init_seeded(nb_sim* sim, int seeder, uint64_t seed, float scale, size_t n, nb_particle* records_out);
size_t nb_count(const nb_sim* sim);

/* INBodySim::Update(dt) (src/Sim/BruteForceCPU.cpp:45-74, src/Sim/BarnesHut.cpp:44-96):
 * nsteps kick-drift steps of size dt, asynchronous on the handle's stream
 * (nb_synchronize waits; reads below synchronise). */
int  nb_step(nb_sim* sim, float dt, int nsteps);
int  nb_synchronize(nb_sim* sim);

/* Writes Position, Velocity and Forces back into n reference records, as
 * Update leaves them: Forces are zero after a direct-sum step
 * (src/Sim/BruteForceCPU.cpp:72) and hold the last Barnes-Hut force otherwise
 * (src/Sim/BarnesHut.cpp:81-95). Colour, OriginalColour and Mass are untouched. */
int  nb_write_back(nb_sim* sim, nb_particle* particles, size_t n);
/* 1 when nb_write_back rewrites the caller's records from the GPU directly
 * (whole 104-byte records, see NB_FLAG_STAGED_IO), 0 when it copies 64-byte
 * packed records to a staging buffer and scatters them on the host; -1 for
 * a null handle. */
int  nb_write_back_direct(const nb_sim* sim);

/* Host copies of the state. Any pointer may be NULL. force3 is the force
 * (m * acceleration) of the last force evaluation. */
int  nb_read_state(nb_sim* sim, float* pos3, double* vel3, double* force3);
/* Evaluates forces at the current positions without stepping and returns
 * them (n x 3 doubles, force on each body). */
int  nb_compute_forces(nb_sim* sim, double* force3);
/* Interactions evaluated by the last force evaluation (pairwise + monopole). */
int  nb_last_interactions(nb_sim* sim, uint64_t* interactions);

/* FP64 direct-sum oracle on the GPU for m sampled target bodies against all n
 * sources, with the handle's law, G and softening (force on each target). */
int  nb_fp64_forces(nb_sim* sim, const int32_t* targets, size_t m, double* force3);
/* half_kick_dt != 0: velocities are synchronised to the positions first,
 * v + a(x) * half_kick_dt (pass dt/2 after kick-drift steps of size dt). */
int  nb_diagnostics(nb_sim* sim, float half_kick_dt, nb_diag* out);

/* Stream the handle launches on (cudaStream_t). */
void* nb_stream(nb_sim* sim);

/* ---- Barnes-Hut octree export (Octree, src/Sim/Octree.cpp:16-145) ------- */
/* Morton keys: the concatenated 3-bit octant path a body takes from the root
 * in Octree::Add, octant = x + 2y + 4z (src/Sim/Octree.cpp:25-41), max_depth
 * levels, the first level in the most significant bits.  depth[i] = levels
 * descended (max_depth for a body in the tree; 0 and key ~0 for a body outside
 * the root cube, which the reference drops but counts).  Keys are those of
 * the current positions. */
int  nb_tree_keys(nb_sim* sim, uint64_t* keys, int32_t* depth);
/* Nodes of the tree of the current positions.  Every non-empty node is one
 * record; the non-empty children of an internal node are consecutive records
 * in octant order starting at first_child (the reference also creates the
 * empty siblings, which hold no body and no mass).  Record 0 is the root. */
typedef struct nb_tree_node {
    int32_t level;        /* 0 = root */
    int32_t count;        /* NumParticles: bodies in the subtree                */
    int32_t first_child;  /* record of the first non-empty child, -1 for a leaf */
    int32_t body;         /* body index of a one-body leaf, else -1             */
    uint64_t prefix;      /* octant path of the node (3*level bits)              */
    double  mass;         /* TotalMass                                           */
    float   com[3];       /* CentreOfMass                                        */
    float   side;         /* Bounds.BottomRight.x - Bounds.TopLeft.x             */
    float   lo[3];        /* Bounds.TopLeft                                      */
    int32_t bucket_begin; /* leaf at the depth cap holding > 1 body: its range  */
    int32_t bucket_end;   /* in nb_tree_order's sorted order, else -1           */
} nb_tree_node;
int  nb_tree_size(nb_sim* sim, size_t* nodes);
int  nb_tree_nodes(nb_sim* sim, nb_tree_node* nodes, size_t capacity);
int  nb_tree_order(nb_sim* sim, int32_t* order);   /* body index at each sorted position */
/* stats8: bodies in the root cube, internal nodes, node records, bodies whose
 * path met a gap between float child bounds (keys and topology are exact
 * when this is 0), depth-cap buckets whose bodies differ (the reference would
 * split them further), failed internal lookups (always 0), bodies outside
 * the root cube, 0. */
int  nb_tree_stats(nb_sim* sim, int64_t* stats8);

/* ---- measurement ---------------------------------------------------------- */
/* Per-phase GPU time measured with CUDA events recorded on the handle's
 * stream around each phase's kernels (enable before the region to measure). */
#define NB_PHASE_DIRECT_FORCE   0   /* K1 direct-sum force kernel                    */
#define NB_PHASE_DIRECT_UPDATE  1   /* K7 partial fold + kick-drift                  */
#define NB_PHASE_KEYS           2   /* K2 Morton keys                                */
#define NB_PHASE_SORT           3   /* K3 radix sort                                 */
#define NB_PHASE_TOPOLOGY       4   /* K4 octree topology                            */
#define NB_PHASE_MASS           5   /* K5 bottom-up mass / centre of mass            */
#define NB_PHASE_TRAVERSE       6   /* K6 tree traversal                             */
#define NB_PHASE_UPDATE         7   /* kick-drift after a tree force pass            */
#define NB_PHASE_COUNT          10
int  nb_profile_enable(nb_sim* sim, int on);      /* on != 0 clears the totals */
/* Total milliseconds and launches of a phase since enabling (synchronises). */
int  nb_profile_read(nb_sim* sim, int phase, double* total_ms, uint64_t* launches);
/* Launch tuning of a handle's kernels (results are unchanged up to FP32
 * summation order).  Keys: "direct_block" (64, 128, 256 threads),
 * "direct_ipt" (1, 2, 4, 8 target bodies per thread), "direct_splits"
 * (source ranges per target block, 0 = automatic), "wait_polls" (polls of
 * each source-tile wait of the direct-sum force kernel before the step is
 * abandoned, 0..4194304, default 4194304; lower values exist only to test the
 * timeout path: the step then leaves the state unchanged and the next
 * nb_synchronize returns NB_ETIMEOUT).  Returns NB_EINVAL for an unknown key
 * or value. */
int  nb_tune(nb_sim* sim, const char* key, int value);
int  nb_get_tune(nb_sim* sim, const char* key, int* value);
/* Kernel launches issued by this handle since creation. */
int  nb_launch_count(nb_sim* sim, uint64_t* launches);
/* Measured FP32 FMA throughput of the device (TFLOP/s, 2 flops per FMA) from
 * a dependent-chain FMA kernel filling every SM, timed with CUDA events. */
int  nb_probe_fp32_peak(int device, double* tflops);
/* The same with the packed FP32x2 FMA (FFMA2) of sm_100+, 4 flops per lane. */
int  nb_probe_fp32x2_peak(int device, double* tflops);

/* ---- batched form: many independent galaxies, one launch per phase ------- */
/* Galaxies with n >= bh_threshold use a group-wise Barnes-Hut (tight cube per
 * galaxy, opening test side / distance(group box, COM) < bh_theta, monopole +
 * quadrupole cells, leaf buckets of leaf_size bodies); the others use the
 * direct sum.  Every phase is one launch over all galaxies, and a step is
 * replayed from a captured CUDA graph.  Parity is the force error against the
 * FP64 direct sum (<= 1e-3), not the reference's per-body opening rule. */
typedef struct nb_batch nb_batch;
typedef struct nb_tuning {
    int direct_block;     /* threads per block of the direct-sum kernel (64, 128, 256) */
    int direct_ipt;       /* target bodies per thread (1, 2; block * ipt <= 256)       */
    int direct_jtile;     /* source bodies per work unit (multiple of 128)             */
    int leaf_size;        /* bodies per Barnes-Hut leaf bucket (1..64)                  */
    int traverse_block;   /* threads per block of the traversal kernel (128)           */
} nb_tuning;
/* base: law, G, softening2, pos_scale, device, stream of the batch. */
int  nb_batch_create(const nb_params* base, size_t bh_threshold, double bh_theta, nb_batch** out);
int  nb_batch_destroy(nb_batch* b);
const char* nb_batch_last_error(const nb_batch* b);
/* Adds one galaxy (host buffers n x float4 each, 1 <= n <= 16 Mi = 16,777,216);
 * galaxy receives its index. */
int  nb_batch_add(nb_batch* b, const float* pos_mass4, const float* vel4, size_t n, int32_t* galaxy);
/* Adds one galaxy that nb_batch_commit generates on the device, straight into
 * the batch's arrays (no host buffers): model 0 exponential disk + 10%
 * Hernquist bulge (nb_seed_disk's defaults), 1 Plummer sphere
 * (nb_seed_plummer's defaults), 2 two Plummer spheres on a parabolic orbit
 * (nb_seed_collision's defaults); 2 <= n <= 16 Mi.  The bodies are those of
 * the host generator of the same (model, seed, n) up to the rounding of the
 * device math functions and of the centre-of-mass sum; a galaxy is the same
 * in every batch and on every run.  The step before the path in the
 * reference: its seeders fill the particle vector on the host
 * (src/Sim/GalaxySeeder.cpp:43-144). */
int  nb_batch_add_generated(nb_batch* b, int model, uint64_t seed, size_t n, int32_t* galaxy);
/* Uploads (or generates) every galaxy, lays out the tables and sizes the tree
 * buffers. */
int  nb_batch_commit(nb_batch* b);
int  nb_batch_set_tuning(nb_batch* b, const nb_tuning* t);
/* Far field of the group traversal: accepted cells far from a group act
 * through the group's third-order local expansion at its centre instead of
 * once per body.  Geometric rule (a state's first evaluation, or alpha 0): a
 * cell farther from the centre than (group half-diagonal / eta) joins it;
 * default eta = 0.2, 0 turns the rule off. */
int  nb_batch_set_far_field(nb_batch* b, double eta);
/* Relative rule of the far field, used once a group's bodies have
 * accelerations from an earlier evaluation (a previous step, or a previous
 * batch for a served job): a cell of mass m at distance r joins when
 * m / r^2 (h / r)^4 < alpha |a|_min / G, h the group's half-diagonal and
 * |a|_min its bodies' smallest acceleration, and h / r < eta_max.  alpha 0
 * turns the rule off (the geometric rule decides every evaluation). */
int  nb_batch_set_far_accuracy(nb_batch* b, double alpha, double eta_max);
int  nb_batch_get_tuning(nb_batch* b, nb_tuning* t);
/* Project autotuner: times candidate leaf sizes, then candidate direct-sum
 * tilings, for trial_steps graph replays each (state restored after each
 * trial) and keeps the fastest. */
int  nb_batch_autotune(nb_batch* b, float dt, int trial_steps);
/* nsteps kick-drift steps of every galaxy, replayed from a captured CUDA graph.
 * The octree's arrays are sized at commit to twice the counts then; steps whose
 * tree outgrows them leave the state unchanged on the device, and the call sizes
 * the tree from the current state and runs those steps again before it returns. */
int  nb_batch_step(nb_batch* b, float dt, int nsteps);
/* After nb_batch_step returned NB_ENOMEM because the octree kept outgrowing
 * its arrays: how many of the nsteps requested were not run (they are the
 * last ones; the state is nsteps - *steps steps ahead of where the call found
 * it).  0 after a call that succeeded. */
int  nb_batch_steps_not_run(nb_batch* b, int* steps);
int  nb_batch_read(nb_batch* b, int32_t galaxy, float* pos_mass4, float* vel4);
/* Forces (n x 3 doubles) of one galaxy at the current state. */
int  nb_batch_forces(nb_batch* b, int32_t galaxy, double* force3);
int  nb_batch_info(nb_batch* b, size_t* galaxies, size_t* bodies, uint64_t* interactions_last);
/* Kernel launches of this batch so far (each graph replay counts its kernels). */
int  nb_batch_launch_count(nb_batch* b, uint64_t* launches);
/* Forest of the last step: stats4 = {traversal groups, internal nodes, cells,
 * Barnes-Hut bodies}. */
int  nb_batch_tree_stats(nb_batch* b, int64_t* stats4);
/* Whole-batch state transfer, galaxies in index order concatenated (the sum
 * of their n bodies x float4): upload from / download to host buffers.  A
 * written state may need a larger octree; the next step sizes it.  Writing a
 * state drops the accelerations of the previous one: its first evaluation
 * takes the far field's geometric rule, as after nb_batch_commit. */
int  nb_batch_write_state(nb_batch* b, const float* pos_mass4, const float* vel4);
int  nb_batch_read_state(nb_batch* b, float* pos_mass4, float* vel4);
void* nb_batch_stream(nb_batch* b);

/* ---- served form: continuous batching of galaxy jobs ---------------------- */
/* Jobs arrive, wait in a FIFO queue, are admitted while the estimated device
 * bytes of the active jobs (640 bytes per body: state, sort and topology
 * scratch, tree cells with quadrupoles at twice their measured count)
 * stay within memory_budget, their bodies within 96 Mi (the batched octree's
 * cell-index range) and a slot is free, and are stepped together in
 * rounds by the batched form; a round takes at most steps_per_round steps,
 * never more than the nearest job completion and, with round_seconds > 0
 * (default 0.1), no more than fit in round_seconds at the batch's measured
 * time per step (one step in the first round of each new batch), so that
 * finished jobs leave and queued ones enter between rounds.  A job keeps its state on the device for
 * its whole life (moved device to device when the batch is rebuilt), so its
 * result does not depend on the jobs it shared rounds with. */
typedef struct nb_server nb_server;
typedef struct nb_server_params {
    nb_params base;           /* law, G, softening2, theta (Barnes-Hut), device     */
    size_t   memory_budget;   /* bytes of device memory the active jobs may hold    */
    int      max_active;      /* slots: jobs stepped together                       */
    int      steps_per_round; /* steps per scheduling round                         */
    size_t   bh_threshold;    /* n >= this: Barnes-Hut, else direct sum             */
    double   round_seconds;   /* a round also stops after about this much stepping
                                 (from the measured time per step; 0: no limit), so
                                 that arriving jobs join soon                       */
} nb_server_params;
typedef struct nb_job {
    uint64_t seed;
    size_t   n;
    int      steps;
    float    dt;              /* jobs are stepped in rounds with the dt of the active jobs */
    int      model;           /* 0 disk + 10% bulge (nb_seed_disk defaults), 1 Plummer   */
} nb_job;
typedef struct nb_job_status {
    uint64_t id;
    int      state;           /* 0 queued, 1 active, 2 done, -1 rejected           */
    int      steps_done;
    double   submit_s, admit_s, done_s;  /* server clock, seconds                  */
    size_t   bytes;           /* estimated device bytes while active               */
} nb_job_status;
int  nb_server_default_params(nb_server_params* p);
int  nb_server_create(const nb_server_params* p, nb_server** out);
int  nb_server_destroy(nb_server* s);
const char* nb_server_last_error(const nb_server* s);
/* Queues a job; its initial conditions are generated on the device, straight
 * into the batch's arrays, when it is admitted (nb_batch_add_generated).  A job
 * of more than 16 Mi bodies (the batched form's galaxy limit) or of more
 * estimated bytes than memory_budget can never run: it is recorded with
 * state -1 (rejected) and the call returns NB_OK. */
int  nb_server_submit(nb_server* s, const nb_job* job, uint64_t* id);
/* One scheduling round: retire finished jobs (final state kept on the host),
 * admit queued jobs that fit the budget and the free slots, step the active
 * jobs.  Returns the active and queued counts. */
int  nb_server_tick(nb_server* s, int* active, int* queued);
double nb_server_clock(nb_server* s);
int  nb_server_status(nb_server* s, uint64_t id, nb_job_status* out);
/* Copies a finished job's final state (n x float4 each) to the host. */
int  nb_server_result(nb_server* s, uint64_t id, float* pos_mass4, float* vel4, size_t n);
/* Forgets a finished (or rejected) job and frees its host copy of the result;
 * a serving loop calls it once the result has been taken, so that the server's
 * memory does not grow with the number of jobs served. */
int  nb_server_release(nb_server* s, uint64_t id);
/* Body-steps completed and rounds run since creation. */
int  nb_server_stats(nb_server* s, uint64_t* body_steps, uint64_t* rounds);
/* Where the server's time went: batch rebuilds (count, seconds: new batch,
 * hand-over, upload, tree sizing), stepping (seconds, steps of the batch, kernel
 * launches of those steps), and host generation of initial conditions
 * (seconds; always 0: jobs are generated on the device, inside the
 * rebuilds). Any pointer may be NULL.  A round that returned NB_ENOMEM
 * because the octree kept outgrowing its arrays counts only the steps it
 * ran, in the jobs' steps_done as here. */
int  nb_server_timing(nb_server* s, uint64_t* rebuilds, double* rebuild_s, uint64_t* batch_steps, double* step_s,
                      double* generate_s, uint64_t* step_launches);

/* ---- allocation-free direct sum -------------------------------------------- */
/* No counterpart in the reference.  For callers that must not allocate device
 * memory while they step: a render loop held to a fixed device-memory budget,
 * a host whose buffers come from its own allocator, or a thread that must
 * not stall (cudaFree synchronises the whole device).
 *
 * Accelerations of n bodies by direct summation (the handle path's kernels:
 * Kahan-compensated FP32), enqueued on `stream` (cudaStream_t, NULL = the
 * default stream) of the current device; nothing is allocated and nothing is
 * read back.  pos_mass4: device buffer of n x (x, y, z, m); accel4: device
 * buffer of n x (ax, ay, az, 0), G applied; both 16-byte aligned.  law:
 * NB_LAW_*; softening2 = eps^2.
 *
 * Working memory: one fixed array of about 18 MB in every GPU's memory from
 * the moment the library's kernels load there until the process exits.  It
 * bounds n to NB_NOALLOC_MAX_BODIES; a larger n returns NB_EINVAL and
 * enqueues nothing.  The first call on a device looks up the array's device
 * address (once per device, with that device current); make that first call
 * before any stream capture.  All calls on a device share the array, so calls
 * whose work overlaps on the GPU (different streams, no ordering between
 * them) race and give undefined results; calls on one stream are ordered.
 * If a bounded device wait inside the kernels runs out, accel4 is filled
 * with NaN. */
#define NB_NOALLOC_MAX_BODIES 65536
int  nb_direct_accel_noalloc(const float* pos_mass4, size_t n, float* accel4, double G, double softening2,
                             int law, void* stream);

/* Headless render hand-off: fills n render vertices (LWParticle) with the
 * current positions and the given per-body colour (n x float4) and scale. */
int  nb_render_vertices(nb_sim* sim, const float* colour4, float scale, nb_render_vertex* out, size_t n);
/* Render hand-off without the per-frame copy of the records
 * (src/States/Simulation/SimulationState.cpp:57-60, 88-103): attaches a device
 * buffer of n vertices (colour4: n x float4 host colours, null for white) that
 * every following kick-drift fills in its epilogue with the moved positions.
 * *device_vertices stays valid until nb_render_detach, the next nb_init_* or
 * nb_destroy; a renderer binds it directly (e.g. through graphics interop or
 * a device copy). nb_render_read copies it to the host. */
int  nb_render_attach(nb_sim* sim, const float* colour4, float scale, void** device_vertices);
int  nb_render_detach(nb_sim* sim);
int  nb_render_read(nb_sim* sim, nb_render_vertex* out, size_t n);

/* ---- initial conditions (seeders) ---------------------------------------- */
/* Counter-based seeded generators. Output: n x (x,y,z,m) and n x (vx,vy,vz,0),
 * host buffers. Every mass is float-representable. */
int  nb_seed_plummer(uint64_t seed, size_t n, double total_mass, double a,
                     float* pos_mass4, float* vel4);
/* Exponential disk (scale length rd, sech^2 height z0, mass fraction
 * 1-bulge_frac) plus Hernquist bulge (scale ab), circular velocities with a
 * Gaussian dispersion of `dispersion` times the circular speed. */
int  nb_seed_disk(uint64_t seed, size_t n, double total_mass, double rd, double z0,
                  double bulge_frac, double ab, double dispersion,
                  float* pos_mass4, float* vel4);
/* Two equal Plummer spheres (each mass total_mass/2, scale a) on a parabolic
 * orbit with pericentre `pericentre`, starting `separation` apart, in the
 * centre-of-mass frame. */
int  nb_seed_collision(uint64_t seed, size_t n, double a, double separation,
                       double pericentre, float* pos_mass4, float* vel4);
/* The reference's own seeders (src/Sim/IParticleSeeder.hpp:12-50), filling
 * reference records: 0 Random (src/Sim/RandomSeeder.cpp:12-40), 1 Galaxy
 * (src/Sim/GalaxySeeder.cpp:43-144), 2 StarSystem
 * (src/Sim/StarSystemSeeder.cpp:17-55), in the reference's units.  The
 * distributions follow the reference; the random streams cannot
 * (std::default_random_engine is implementation-defined). */
int  nb_seed_reference(int seeder, uint64_t seed, float scale, nb_particle* out, size_t n);

/* ---- .nbody files (src/States/Simulation/SimulationState.cpp:229-332) ---- */
/* Raw little-endian nb_particle records.  nb_file_read stores the record
 * count in *n (pass particles = NULL to query it) and, like
 * InitParticlesFromFile, re-centres the positions on the centre of mass when
 * recentre != 0. */
int  nb_file_write(const char* path, const nb_particle* particles, size_t n);
int  nb_file_read(const char* path, nb_particle* particles, size_t capacity, size_t* n, int recentre);
#ifdef __cplusplus
}
#endif
#endif /* NBODY_GB300_H */
