/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A C entry surface over the reference's own CPU N-body code, compiled from
 * its unmodified sources (src/Sim/Octree.cpp, src/Sim/BarnesHut.cpp,
 * src/Sim/BruteForceCPU.cpp with src/Sim/Physics.hpp, src/Core/Vec3.hpp,
 * src/Core/ThreadPool.hpp, src/Render/Misc/Particle.hpp) against the
 * type-only headers in oracle/ref/shim.  The tests use it to pin the oracle
 * (oracle/nb_oracle.cpp) and to generate golden vectors; nothing in the
 * product links it, and it is built only where the reference sources exist.
 *
 * Entry points:
 *   ref_workers()          worker count of the reference's CThreadPool here
 *                          (src/Core/ThreadPool.hpp:39-51)
 *   ref_octree_build()     Octree over BarnesHut's +-4000 cube, Add in array
 *                          order, CalculateMass (src/Sim/BarnesHut.cpp:14-21,46-56)
 *   ref_octree_export()    every node, depth-first in octant order
 *   ref_octree_forces()    Octree::CalculateForce per target (src/Sim/Octree.cpp:107-145)
 *   ref_bh_update()        BarnesHut::Update (src/Sim/BarnesHut.cpp:44-96)
 *   ref_bf_update()        BruteForceCPU::Update (src/Sim/BruteForceCPU.cpp:45-74)
 * Physics constants are the reference's (src/Sim/Physics.hpp:9-17):
 * G = 6.674e-11, S = 10, StarSystemScale = 2.3e13.
 */
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <functional>
#include <list>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

// The node export reads Octree's private members (children, leaf flag, body
// pointer): this translation unit sees them as public.  The class layout is
// the same either way.
#define private public
#include "Sim/Octree.hpp"
#undef private
#include "Sim/BarnesHut.hpp"
#include "Sim/BruteForceCPU.hpp"

static_assert(sizeof(Particle) == 104, "the reference record must be 104 bytes here too");

namespace {

struct RefTree {
    std::vector<Particle> particles;
    std::unique_ptr<Octree> root;
};

struct NodeOut {
    int32_t* ints;       // depth, NumParticles, IsLeaf, body
    uint64_t* prefix;    // octant path, 3 bits per level
    double* mass;        // TotalMass
    float* floats;       // CentreOfMass xyz, TopLeft xyz, BottomRight xyz, Size
    size_t k;
    const Particle* base;
};

size_t count_nodes(const Octree* o) {
    size_t c = 1;
    if (!o->IsLeaf)
        for (const auto& ch : o->Children) c += count_nodes(ch.get());
    return c;
}

void export_nodes(const Octree* o, uint64_t prefix, NodeOut& out) {
    const size_t k = out.k++;
    out.ints[4 * k + 0] = o->Depth;
    out.ints[4 * k + 1] = o->NumParticles;
    out.ints[4 * k + 2] = o->IsLeaf ? 1 : 0;
    out.ints[4 * k + 3] = (o->NumParticles == 1 && o->P) ? (int32_t)(o->P - out.base) : -1;
    out.prefix[k] = prefix;
    out.mass[k] = o->TotalMass;
    float* f = out.floats + 10 * k;
    f[0] = o->CentreOfMass.x; f[1] = o->CentreOfMass.y; f[2] = o->CentreOfMass.z;
    f[3] = o->Bounds.TopLeft.x; f[4] = o->Bounds.TopLeft.y; f[5] = o->Bounds.TopLeft.z;
    f[6] = o->Bounds.BottomRight.x; f[7] = o->Bounds.BottomRight.y; f[8] = o->Bounds.BottomRight.z;
    f[9] = o->Size;
    if (!o->IsLeaf)
        for (int c = 0; c < 8; ++c) export_nodes(o->Children[c].get(), (prefix << 3) | (uint64_t)c, out);
}

int max_depth(const Octree* o) {
    int d = o->Depth;
    if (!o->IsLeaf)
        for (const auto& ch : o->Children) d = std::max(d, max_depth(ch.get()));
    return d;
}

// The simulators own worker threads that never exit (the reference's pool
// detaches them); one instance of each is kept for the life of the process.
BarnesHut* bh_sim() {
    static BarnesHut* s = new BarnesHut(nullptr);
    return s;
}
BruteForceCPU* bf_sim() {
    static BruteForceCPU* s = new BruteForceCPU(nullptr);
    return s;
}
std::mutex g_lock;

}  // namespace

extern "C" {

int ref_workers(void) {
    unsigned hc = std::thread::hardware_concurrency();
    return (int)(hc == 0 ? 8 : hc) - 1;
}

void* ref_octree_build(const void* records, size_t n) {
    auto* t = new RefTree();
    t->particles.resize(n);
    std::memcpy(t->particles.data(), records, n * sizeof(Particle));
    const float size = 4000.0f;   // BarnesHut's root cube (src/Sim/BarnesHut.cpp:14-21)
    BoundingCube bounds = {{-size, -size, -size}, {+size, +size, +size}};
    t->root = std::make_unique<Octree>(bounds);
    Particle* p = t->particles.data();
    for (size_t i = 0; i < n; ++i) t->root->Add(p + i);
    t->root->CalculateMass();
    return t;
}

void ref_octree_free(void* h) { delete (RefTree*)h; }

size_t ref_octree_node_count(void* h) { return count_nodes(((RefTree*)h)->root.get()); }

int ref_octree_max_depth(void* h) { return max_depth(((RefTree*)h)->root.get()); }

int ref_octree_export(void* h, int32_t* ints4, uint64_t* prefix, double* mass, float* floats10) {
    RefTree* t = (RefTree*)h;
    NodeOut out{ints4, prefix, mass, floats10, 0, t->particles.data()};
    export_nodes(t->root.get(), 0, out);
    return 0;
}

int ref_octree_forces(void* h, const int32_t* targets, size_t m, double theta, double* force3) {
    std::lock_guard<std::mutex> g(g_lock);   // Octree::Theta is a global
    RefTree* t = (RefTree*)h;
    Octree::Theta = theta;
    for (size_t k = 0; k < m; ++k) {
        Vec3d f = t->root->CalculateForce(&t->particles[(size_t)targets[k]]);
        force3[3 * k] = f.x; force3[3 * k + 1] = f.y; force3[3 * k + 2] = f.z;
    }
    return 0;
}

int ref_bh_update(void* records, size_t n, float dt, double theta, int steps) {
    std::lock_guard<std::mutex> g(g_lock);
    std::vector<Particle> v(n);
    std::memcpy(v.data(), records, n * sizeof(Particle));
    Octree::Theta = theta;
    BarnesHut* s = bh_sim();
    s->Init(v);
    for (int k = 0; k < steps; ++k) s->Update(dt);
    std::memcpy(records, v.data(), n * sizeof(Particle));
    return 0;
}

int ref_bf_update(void* records, size_t n, float dt, int steps) {
    std::lock_guard<std::mutex> g(g_lock);
    std::vector<Particle> v(n);
    std::memcpy(v.data(), records, n * sizeof(Particle));
    BruteForceCPU* s = bf_sim();
    s->Init(v);
    for (int k = 0; k < steps; ++k) s->Update(dt);
    std::memcpy(records, v.data(), n * sizeof(Particle));
    return 0;
}

}  // extern "C"
