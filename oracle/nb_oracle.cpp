/*
 * nb_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference simulator's N-body step, used as the
 * checker for the CUDA path (tests, __graft_entry__.smoke, and the CPU
 * baseline leg of bench.py).  Nothing in the product library links or calls
 * this file.
 *
 * Pinned to the reference's own code: the reference (Procedural-Universe)
 * holds no tests or golden vectors for this path, but its CPU simulator
 * sources compile unmodified against type-only stand-ins for the DirectXTK
 * and Direct3D headers (oracle/ref/Makefile), and this restatement is
 * bit-identical to that build on every octree node, force and updated
 * record (tests/test_reference_pin_cpu.py), apart from the two deviations
 * below that change results (1 and 2).  The SimpleMath arithmetic stays
 * unpinned: both sides compute it as the plain float operations below.
 *
 * Restated reference code:
 *   Phys::Gravity          src/Sim/Physics.hpp:25-47
 *   BruteForceCPU          src/Sim/BruteForceCPU.cpp:25-74
 *   BarnesHut::Update      src/Sim/BarnesHut.cpp:44-110
 *   Octree                 src/Sim/Octree.hpp:13-49, src/Sim/Octree.cpp:1-145
 *   CThreadPool partition  src/Core/ThreadPool.hpp:39-51
 *   struct Particle        src/Render/Misc/Particle.hpp:8-18
 * DirectXTK SimpleMath vector ops (third-party, not vendored, version not
 * recoverable) are restated from its published behaviour as plain float
 * arithmetic: Length = sqrtf((x*x + y*y) + z*z); Normalize = v / Length
 * (zero stays zero); DistanceSquared = the same dot of the difference;
 * Vector3 / s = Vector3 * (1.f / s).
 *
 * Deliberate deviations, each documented:
 *   1. The remainder slice of the thread partition covers the tail bodies
 *      (the reference recomputes [T*rem, (T+1)*rem) for direct sum and
 *      [T, T+rem) for Barnes-Hut, leaving tail bodies without force).
 *   2. The octree stops splitting at max_depth (default 21 = 63-bit keys);
 *      a leaf at the cap holds a bucket of bodies.  A bucket's mass and
 *      centre of mass sum its bodies in ascending index order; an opened
 *      bucket contributes the pairwise force of each member other than the
 *      target.  The reference recurses without limit (forever for
 *      coincident bodies).
 *   3. G, S (= eps^2), the drift divisor (StarSystemScale) and the root
 *      half-width are parameters instead of constants.
 * Build with -ffp-contract=off so that float arithmetic rounds exactly as
 * written (no fused multiply-add), on x86-64 and aarch64 alike.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <cstddef>
#include <vector>
#include <thread>
#include <algorithm>
#include <functional>

namespace {

struct Particle {              /* src/Render/Misc/Particle.hpp:8-18 */
    float  pos[3];
    float  colour[4];
    float  ocolour[4];
    float  pad;
    double vel[3];
    double force[3];
    double mass;
};
static_assert(sizeof(Particle) == 104, "Particle record must be 104 bytes");
static_assert(offsetof(Particle, vel) == 48, "Velocity at 48");
static_assert(offsetof(Particle, force) == 72, "Forces at 72");
static_assert(offsetof(Particle, mass) == 96, "Mass at 96");

/* SimpleMath restatement (float, evaluation order as written). */
static inline float dot3(const float a[3]) { return (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]; }
static inline float dist2(const float a[3], const float b[3]) {
    float d[3] = { b[0] - a[0], b[1] - a[1], b[2] - a[2] };
    return dot3(d);
}
static inline void normalize3(float v[3]) {
    float len = sqrtf(dot3(v));
    if (len > 0.0f) { v[0] = v[0] / len; v[1] = v[1] / len; v[2] = v[2] / len; }
    else { v[0] = v[1] = v[2] = 0.0f; }
}

/* Phys::Gravity(a, b) (src/Sim/Physics.hpp:25-35): -(G*ma*mb)/(d2+S), d2 in float. */
static inline double gravity(double G, double S, double ma, double mb, const float pa[3], const float pb[3]) {
    double d = (double)dist2(pa, pb);
    return -(G * ma * mb) / (d + S);
}

struct Laws { double G, S; int law; };

/* Pairwise force on target t from source s in the reference form
 * F = f * normalize(pt - ps). Returns it in out[3]. */
static inline void pair_force_ref(const Laws& L, double mt, double ms, const float pt[3], const float ps[3],
                                  bool source_first, double out[3]) {
    /* BruteForceCPU calls Gravity(a=source j, b=target i): (G*mj)*mi.
     * Octree::CalculateForce calls Gravity(*p=target, *P=source): (G*mt)*ms. */
    double f = source_first ? gravity(L.G, L.S, ms, mt, ps, pt) : gravity(L.G, L.S, mt, ms, pt, ps);
    float diff[3] = { pt[0] - ps[0], pt[1] - ps[1], pt[2] - ps[2] };
    normalize3(diff);
    out[0] = f * diff[0]; out[1] = f * diff[1]; out[2] = f * diff[2];
}

/* Plummer law in the same shape: F = -G mt ms (pt-ps) / (r^2+S)^{3/2}, r^2 in float. */
static inline void pair_force_plummer(const Laws& L, double mt, double ms, const float pt[3], const float ps[3],
                                      double out[3]) {
    float diff[3] = { pt[0] - ps[0], pt[1] - ps[1], pt[2] - ps[2] };
    double r2 = (double)dot3(diff) + L.S;
    double f = -(L.G * mt * ms) / (r2 * std::sqrt(r2));
    out[0] = f * diff[0]; out[1] = f * diff[1]; out[2] = f * diff[2];
}

static inline void pair_force(const Laws& L, double mt, double ms, const float pt[3], const float ps[3],
                              bool source_first, double out[3]) {
    if (L.law == 0) pair_force_ref(L, mt, ms, pt, ps, source_first, out);
    else pair_force_plummer(L, mt, ms, pt, ps, out);
}

/* CThreadPool partition (src/Core/ThreadPool.hpp:39-51, src/Sim/BruteForceCPU.cpp:45-59):
 * T workers each take N/T consecutive bodies; the caller's thread runs the
 * remainder -- here the true tail (deviation 1). */
static void parallel_slices(size_t n, int nthreads, const std::function<void(size_t, size_t)>& fn) {
    if (nthreads <= 0) {
        unsigned hc = std::thread::hardware_concurrency();
        nthreads = (int)(hc == 0 ? 8 : hc) - 1;
        if (nthreads < 1) nthreads = 1;
        if (nthreads > 31) nthreads = 31;
    }
    size_t per = n / (size_t)nthreads;
    size_t rem = n % (size_t)nthreads;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) {
        size_t b = (size_t)t * per, e = b + per;
        if (e > b) th.emplace_back(fn, b, e);
    }
    if (rem > 0) fn((size_t)nthreads * per, n);
    for (auto& x : th) x.join();
}

/* ------------------------------------------------------------------------ */
/* Octree (src/Sim/Octree.hpp:13-49, src/Sim/Octree.cpp)                    */
/* Nodes live in an arena; children of a split node are 8 consecutive      */
/* entries in octant order i = x + 2y + 4z.                                 */
/* ------------------------------------------------------------------------ */
struct Node {
    int    depth = 0;
    int    num = 0;          /* NumParticles (counts dropped bodies too) */
    float  tl[3] = {0, 0, 0};
    float  br[3] = {0, 0, 0};
    double mass = 0.0;       /* TotalMass */
    float  com[3] = {0, 0, 0};
    bool   leaf = true;      /* IsLeaf */
    float  size = 0.0f;      /* Size = BottomRight.x - TopLeft.x */
    int    P = -1;           /* body of a one-body leaf */
    int    child = -1;       /* index of child 0 */
    std::vector<int> bucket; /* bodies of a leaf at the depth cap (deviation 2) */
    uint64_t prefix = 0;     /* octant path, 3 bits per level */
};

struct Tree {
    std::vector<Node> nodes;
    const float* pos = nullptr;    /* n x 3 */
    const double* mass = nullptr;  /* n */
    int max_depth = 21;
    std::vector<uint64_t> keys;    /* octant path per body */
    std::vector<int> body_depth;   /* levels descended per body */
    long long deeper_buckets = 0;  /* buckets the reference would split further */

    /* BoundingCube::Contains (src/Sim/Octree.hpp:18-22): half-open [tl, br). */
    bool contains(const Node& nd, int b) const {
        const float* p = pos + 3 * (size_t)b;
        return p[0] >= nd.tl[0] && p[1] >= nd.tl[1] && p[2] >= nd.tl[2] &&
               p[0] < nd.br[0] && p[1] < nd.br[1] && p[2] < nd.br[2];
    }
    bool contains_pt(const Node& nd, const float* p) const {
        return p[0] >= nd.tl[0] && p[1] >= nd.tl[1] && p[2] >= nd.tl[2] &&
               p[0] < nd.br[0] && p[1] < nd.br[1] && p[2] < nd.br[2];
    }

    int make_root(float half) {
        Node r;
        r.tl[0] = r.tl[1] = r.tl[2] = -half;
        r.br[0] = r.br[1] = r.br[2] = +half;
        r.size = r.br[0] - r.tl[0];
        nodes.push_back(r);
        return 0;
    }

    /* Octree::Split (src/Sim/Octree.cpp:16-51): float bounds accumulated as
     * cur += size; the child's Size is recomputed from its bounds. */
    void split(int ni) {
        float size = nodes[ni].size / 2;
        float tl[3] = { nodes[ni].tl[0], nodes[ni].tl[1], nodes[ni].tl[2] };
        int depth = nodes[ni].depth;
        uint64_t prefix = nodes[ni].prefix;
        int first = (int)nodes.size();
        nodes.resize(nodes.size() + 8);
        float cur[3] = { tl[0], tl[1], tl[2] };
        int i = 0;
        for (int z = 0; z < 2; ++z) {
            cur[1] = tl[1];
            for (int y = 0; y < 2; ++y) {
                cur[0] = tl[0];
                for (int x = 0; x < 2; ++x, ++i) {
                    Node& c = nodes[first + i];
                    c.tl[0] = cur[0]; c.tl[1] = cur[1]; c.tl[2] = cur[2];
                    c.br[0] = cur[0] + size; c.br[1] = cur[1] + size; c.br[2] = cur[2] + size;
                    c.size = c.br[0] - c.tl[0];
                    c.depth = depth + 1;
                    c.prefix = (prefix << 3) | (uint64_t)i;
                    cur[0] += size;
                }
                cur[1] += size;
            }
            cur[2] += size;
        }
        nodes[ni].child = first;
        nodes[ni].leaf = false;
    }

    /* Octree::Add (src/Sim/Octree.cpp:53-84), with the depth cap. */
    void add(int ni, int b) {
        if (nodes[ni].num > 1) {
            if (!nodes[ni].bucket.empty() || nodes[ni].depth >= max_depth) {
                nodes[ni].bucket.push_back(b);
            } else {
                int c0 = nodes[ni].child;
                for (int c = 0; c < 8; ++c)
                    if (contains(nodes[c0 + c], b)) add(c0 + c, b);
            }
        } else if (nodes[ni].num == 1) {
            int P = nodes[ni].P;
            if (nodes[ni].depth >= max_depth) {
                nodes[ni].bucket.push_back(P);
                nodes[ni].bucket.push_back(b);
            } else {
                if (nodes[ni].leaf) split(ni);
                int c0 = nodes[ni].child;
                for (int c = 0; c < 8; ++c) {
                    if (contains(nodes[c0 + c], b)) add(c0 + c, b);
                    if (contains(nodes[c0 + c], P)) add(c0 + c, P);
                }
            }
            nodes[ni].P = -1;
        } else {
            nodes[ni].P = b;
        }
        ++nodes[ni].num;
    }

    /* Octree::CalculateMass (src/Sim/Octree.cpp:86-105): TotalMass in
     * double; CentreOfMass += child COM * float(child mass) in float; then
     * scaled by 1/float(TotalMass). */
    void mass_pass(int ni) {
        Node& nd = nodes[ni];
        if (!nd.bucket.empty()) {
            std::vector<int> mem = nd.bucket;
            std::sort(mem.begin(), mem.end());
            double M = 0.0; float c[3] = {0, 0, 0};
            for (int b : mem) {
                M += mass[b];
                float mf = (float)mass[b];
                const float* p = pos + 3 * (size_t)b;
                float t0 = p[0] * mf, t1 = p[1] * mf, t2 = p[2] * mf;
                c[0] = c[0] + t0; c[1] = c[1] + t1; c[2] = c[2] + t2;
            }
            if (M > 0.0) {
                float inv = 1.f / (float)M;
                c[0] = c[0] * inv; c[1] = c[1] * inv; c[2] = c[2] * inv;
            }
            nd.mass = M; nd.com[0] = c[0]; nd.com[1] = c[1]; nd.com[2] = c[2];
            return;
        }
        if (nd.num == 1) {
            const float* p = pos + 3 * (size_t)nd.P;
            nd.com[0] = p[0]; nd.com[1] = p[1]; nd.com[2] = p[2];
            nd.mass = mass[nd.P];
        } else if (!nd.leaf) {
            int c0 = nd.child;
            double M = 0.0; float c[3] = {0, 0, 0};
            for (int k = 0; k < 8; ++k) {
                mass_pass(c0 + k);
                const Node& ch = nodes[c0 + k];
                M += ch.mass;
                float mf = (float)ch.mass;
                float t0 = ch.com[0] * mf, t1 = ch.com[1] * mf, t2 = ch.com[2] * mf;
                c[0] = c[0] + t0; c[1] = c[1] + t1; c[2] = c[2] + t2;
            }
            if (M > 0.0) {
                float inv = 1.f / (float)M;
                c[0] = c[0] * inv; c[1] = c[1] * inv; c[2] = c[2] * inv;
            }
            Node& nd2 = nodes[ni];
            nd2.mass = M; nd2.com[0] = c[0]; nd2.com[1] = c[1]; nd2.com[2] = c[2];
        }
    }

    /* Octree::CalculateForce (src/Sim/Octree.cpp:107-145) for target b.
     * theta_f = smallest float >= Theta, so that float(d/r) < theta_f is the
     * reference's comparison of a float ratio against the double Theta. */
    void force(int ni, int b, const Laws& L, float theta_f, double out[3], long long& inter) const {
        const Node& nd = nodes[ni];
        const float* p = pos + 3 * (size_t)b;
        out[0] = out[1] = out[2] = 0.0;
        if (nd.bucket.empty() && nd.num == 1) {
            if (b != nd.P && !contains(nd, b)) {
                pair_force(L, mass[b], mass[nd.P], p, pos + 3 * (size_t)nd.P, false, out);
                ++inter;
            }
            return;
        }
        float dv[3] = { p[0] - nd.com[0], p[1] - nd.com[1], p[2] - nd.com[2] };
        float r = sqrtf(dot3(dv));
        float d = nd.br[0] - nd.tl[0];
        if (d / r < theta_f) {
            if (nd.num > 0) ++inter;   /* empty nodes contribute exactly zero */
            pair_force(L, mass[b], nd.mass, p, nd.com, false, out);
            return;
        }
        if (!nd.bucket.empty()) {
            std::vector<int> mem = nd.bucket;
            std::sort(mem.begin(), mem.end());
            for (int q : mem) {
                if (q == b) continue;
                double f[3];
                pair_force(L, mass[b], mass[q], p, pos + 3 * (size_t)q, false, f);
                out[0] += f[0]; out[1] += f[1]; out[2] += f[2];
                ++inter;
            }
            return;
        }
        if (!nd.leaf) {
            for (int k = 0; k < 8; ++k) {
                double f[3];
                force(nd.child + k, b, L, theta_f, f, inter);
                out[0] += f[0]; out[1] += f[1]; out[2] += f[2];
            }
        }
    }

    /* Octant path of each body as Add descends (for the key export). */
    void compute_keys(size_t n) {
        keys.assign(n, 0);
        body_depth.assign(n, 0);
        for (size_t b = 0; b < n; ++b) {
            int ni = 0;
            if (!contains(nodes[0], (int)b)) { keys[b] = ~0ull; body_depth[b] = 0; continue; }
            uint64_t key = 0; int depth = 0;
            while (!nodes[ni].leaf) {
                int c0 = nodes[ni].child, found = -1;
                for (int c = 0; c < 8; ++c) if (contains(nodes[c0 + c], (int)b)) { found = c; break; }
                if (found < 0) break;
                key = (key << 3) | (uint64_t)found;
                ++depth; ni = c0 + found;
            }
            /* Continue the path below the leaf with the same Split arithmetic
             * so that every in-tree body gets a full max_depth-level key. */
            Node cur = nodes[ni];
            while (depth < max_depth) {
                float size = cur.size / 2;
                float lo[3] = { cur.tl[0], cur.tl[1], cur.tl[2] };
                float mid[3] = { lo[0] + size, lo[1] + size, lo[2] + size };
                float hi[3] = { mid[0] + size, mid[1] + size, mid[2] + size };
                const float* p = pos + 3 * b;
                int oct = 0; bool ok = true;
                for (int a = 0; a < 3; ++a) {
                    if (p[a] >= mid[a] && p[a] < hi[a]) { oct |= 1 << a; cur.tl[a] = mid[a]; cur.br[a] = hi[a]; }
                    else if (p[a] >= lo[a] && p[a] < mid[a]) { cur.tl[a] = lo[a]; cur.br[a] = mid[a]; }
                    else ok = false;
                }
                if (!ok) break;
                cur.size = cur.br[0] - cur.tl[0];
                key = (key << 3) | (uint64_t)oct;
                ++depth;
            }
            /* a path cut short by a gap between float child bounds keeps its
             * octants left-aligned (the lower levels read as octant 0) */
            if (depth < max_depth) key <<= 3 * (max_depth - depth);
            keys[b] = key; body_depth[b] = depth;
        }
    }
};

struct OracleTree {
    Tree t;
    std::vector<float> pos;
    std::vector<double> mass;
};

} /* namespace */

extern "C" {

/* ---- direct sum ------------------------------------------------------- */

/* BruteForceCPU::Exec (src/Sim/BruteForceCPU.cpp:25-43) over every body:
 * force3[i] = sum over j != i in ascending j of Gravity(j, i) * normalize(pi - pj). */
int orc_direct_forces(const void* particles, size_t n, double G, double S, int law, int nthreads, double* force3) {
    const Particle* P = (const Particle*)particles;
    Laws L{G, S, law};
    parallel_slices(n, nthreads, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double F[3] = {0, 0, 0};
            for (size_t j = 0; j < n; ++j) {
                if (i == j) continue;
                double f[3];
                pair_force(L, P[i].mass, P[j].mass, P[i].pos, P[j].pos, true, f);
                F[0] += f[0]; F[1] += f[1]; F[2] += f[2];
            }
            force3[3 * i + 0] = F[0]; force3[3 * i + 1] = F[1]; force3[3 * i + 2] = F[2];
        }
    });
    return 0;
}

/* The same loop for a subset of targets (CPU-baseline sampling). */
int orc_direct_forces_subset(const void* particles, size_t n, const int32_t* targets, size_t m, double G, double S,
                             int law, int nthreads, double* force3) {
    const Particle* P = (const Particle*)particles;
    Laws L{G, S, law};
    parallel_slices(m, nthreads, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; ++k) {
            const size_t i = (size_t)targets[k];
            double F[3] = {0, 0, 0};
            for (size_t j = 0; j < n; ++j) {
                if (i == j) continue;
                double f[3];
                pair_force(L, P[i].mass, P[j].mass, P[i].pos, P[j].pos, true, f);
                F[0] += f[0]; F[1] += f[1]; F[2] += f[2];
            }
            force3[3 * k + 0] = F[0]; force3[3 * k + 1] = F[1]; force3[3 * k + 2] = F[2];
        }
    });
    return 0;
}

/* Kick-drift of BruteForceCPU::Update / BarnesHut::Update
 * (src/Sim/BruteForceCPU.cpp:61-73, src/Sim/BarnesHut.cpp:81-95). */
static void kick_drift(Particle* P, size_t n, float dt, double scale, bool zero_forces) {
    for (size_t i = 0; i < n; ++i) {
        double a[3] = { P[i].force[0] / P[i].mass, P[i].force[1] / P[i].mass, P[i].force[2] / P[i].mass };
        for (int k = 0; k < 3; ++k) P[i].vel[k] += a[k] * (double)dt;
        double v[3] = { (P[i].vel[0] * (double)dt) / scale, (P[i].vel[1] * (double)dt) / scale,
                        (P[i].vel[2] * (double)dt) / scale };
        for (int k = 0; k < 3; ++k) P[i].pos[k] = P[i].pos[k] + (float)v[k];
        if (zero_forces) P[i].force[0] = P[i].force[1] = P[i].force[2] = 0.0;
    }
}

/* BruteForceCPU::Update (src/Sim/BruteForceCPU.cpp:45-74), nsteps times.
 * Forces accumulate onto the records' Forces (zero after each step). */
int orc_direct_step(void* particles, size_t n, double G, double S, int law, double scale, float dt,
                    int nsteps, int nthreads) {
    Particle* P = (Particle*)particles;
    std::vector<double> F(3 * n);
    for (int s = 0; s < nsteps; ++s) {
        orc_direct_forces(particles, n, G, S, law, nthreads, F.data());
        for (size_t i = 0; i < n; ++i) for (int k = 0; k < 3; ++k) P[i].force[k] += F[3 * i + k];
        kick_drift(P, n, dt, scale, true);
    }
    return 0;
}

/* ---- Barnes-Hut --------------------------------------------------------- */

/* Builds the octree of BarnesHut::Update (src/Sim/BarnesHut.cpp:44-56):
 * root cube +-half, serial Add in array order, CalculateMass. */
void* orc_tree_build(const void* particles, size_t n, float half, int max_depth) {
    const Particle* P = (const Particle*)particles;
    OracleTree* ot = new OracleTree();
    ot->pos.resize(3 * n); ot->mass.resize(n);
    for (size_t i = 0; i < n; ++i) {
        ot->pos[3 * i] = P[i].pos[0]; ot->pos[3 * i + 1] = P[i].pos[1]; ot->pos[3 * i + 2] = P[i].pos[2];
        ot->mass[i] = P[i].mass;
    }
    Tree& t = ot->t;
    t.pos = ot->pos.data(); t.mass = ot->mass.data(); t.max_depth = max_depth;
    t.nodes.reserve(4 * n + 16);
    t.make_root(half);
    for (size_t i = 0; i < n; ++i) t.add(0, (int)i);
    t.mass_pass(0);
    t.compute_keys(n);
    /* buckets whose bodies would still be separated by a further split */
    for (const Node& nd : t.nodes) {
        if (nd.bucket.size() < 2) continue;
        const float* p0 = t.pos + 3 * (size_t)nd.bucket[0];
        for (int b : nd.bucket) {
            const float* p = t.pos + 3 * (size_t)b;
            if (p[0] != p0[0] || p[1] != p0[1] || p[2] != p0[2]) { ++t.deeper_buckets; break; }
        }
    }
    return ot;
}

void orc_tree_free(void* h) { delete (OracleTree*)h; }

size_t orc_tree_node_count(void* h) { return ((OracleTree*)h)->t.nodes.size(); }
long long orc_tree_deeper_buckets(void* h) { return ((OracleTree*)h)->t.deeper_buckets; }

/* Node export, in the arena order of the reference's recursion
 * (parents before children, children of a node consecutive). Per node:
 * ints[6] = {level, count, first_child, body, bucket_size, is_leaf},
 * u64 prefix, double mass, floats[7] = {com xyz, side, lo xyz}. */
int orc_tree_nodes(void* h, int32_t* ints6, uint64_t* prefix, double* mass, float* floats7) {
    const Tree& t = ((OracleTree*)h)->t;
    for (size_t i = 0; i < t.nodes.size(); ++i) {
        const Node& nd = t.nodes[i];
        ints6[6 * i + 0] = nd.depth;
        ints6[6 * i + 1] = nd.num;
        ints6[6 * i + 2] = nd.child;
        ints6[6 * i + 3] = (nd.bucket.empty() && nd.num == 1) ? nd.P : -1;
        ints6[6 * i + 4] = (int)nd.bucket.size();
        ints6[6 * i + 5] = nd.leaf ? 1 : 0;
        prefix[i] = nd.prefix;
        mass[i] = nd.mass;
        floats7[7 * i + 0] = nd.com[0]; floats7[7 * i + 1] = nd.com[1]; floats7[7 * i + 2] = nd.com[2];
        floats7[7 * i + 3] = nd.size;
        floats7[7 * i + 4] = nd.tl[0]; floats7[7 * i + 5] = nd.tl[1]; floats7[7 * i + 6] = nd.tl[2];
    }
    return 0;
}

/* Bucket members (sorted by index) of node i; returns the count. */
int orc_tree_bucket(void* h, size_t i, int32_t* out, int cap) {
    const Tree& t = ((OracleTree*)h)->t;
    std::vector<int> mem = t.nodes[i].bucket;
    std::sort(mem.begin(), mem.end());
    int k = 0;
    for (int b : mem) { if (k < cap) out[k] = b; ++k; }
    return k;
}

int orc_tree_keys(void* h, uint64_t* keys, int32_t* depth) {
    const Tree& t = ((OracleTree*)h)->t;
    for (size_t i = 0; i < t.keys.size(); ++i) { keys[i] = t.keys[i]; depth[i] = t.body_depth[i]; }
    return 0;
}

static float theta_float(double theta) {
    /* smallest float >= theta */
    float f = (float)theta;
    if ((double)f < theta) f = std::nextafter(f, INFINITY);
    return f;
}

/* Barnes-Hut forces (src/Sim/BarnesHut.cpp:59-79, 103-110):
 * Forces = Tree->CalculateForce(p) for every body (tail fixed). */
int orc_bh_forces(void* h, double G, double S, int law, double theta, int nthreads, double* force3,
                  long long* interactions) {
    const Tree& t = ((OracleTree*)h)->t;
    Laws L{G, S, law};
    float tf = theta_float(theta);
    size_t n = ((OracleTree*)h)->mass.size();
    std::vector<long long> cnt(n, 0);
    parallel_slices(n, nthreads, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double f[3]; long long c = 0;
            t.force(0, (int)i, L, tf, f, c);
            force3[3 * i] = f[0]; force3[3 * i + 1] = f[1]; force3[3 * i + 2] = f[2];
            cnt[i] = c;
        }
    });
    if (interactions) { long long s = 0; for (auto c : cnt) s += c; *interactions = s; }
    return 0;
}

/* Barnes-Hut forces for a subset of targets (CPU-baseline sampling). */
int orc_bh_forces_subset(void* h, const int32_t* targets, size_t m, double G, double S, int law, double theta,
                         int nthreads, double* force3) {
    const Tree& t = ((OracleTree*)h)->t;
    Laws L{G, S, law};
    float tf = theta_float(theta);
    parallel_slices(m, nthreads, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; ++k) {
            double f[3]; long long c = 0;
            t.force(0, targets[k], L, tf, f, c);
            force3[3 * k] = f[0]; force3[3 * k + 1] = f[1]; force3[3 * k + 2] = f[2];
        }
    });
    return 0;
}

/* BarnesHut::Update (src/Sim/BarnesHut.cpp:44-96), nsteps times.
 * Forces are assigned (not accumulated) and not reset. */
int orc_bh_step(void* particles, size_t n, double G, double S, int law, double theta, double scale,
                float half, int max_depth, float dt, int nsteps, int nthreads) {
    Particle* P = (Particle*)particles;
    std::vector<double> F(3 * n);
    for (int s = 0; s < nsteps; ++s) {
        void* h = orc_tree_build(particles, n, half, max_depth);
        orc_bh_forces(h, G, S, law, theta, nthreads, F.data(), nullptr);
        orc_tree_free(h);
        for (size_t i = 0; i < n; ++i) for (int k = 0; k < 3; ++k) P[i].force[k] = F[3 * i + k];
        kick_drift(P, n, dt, scale, false);
    }
    return 0;
}

/* ---- FP64 direct sum (the exact law in double) --------------------------- */
int orc_fp64_forces(const double* pos3, const double* mass, size_t n, const int32_t* targets, size_t m,
                    double G, double S, int law, int nthreads, double* force3) {
    parallel_slices(m, nthreads, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; ++k) {
            size_t i = (size_t)targets[k];
            double F[3] = {0, 0, 0};
            for (size_t j = 0; j < n; ++j) {
                if (j == i) continue;
                double d[3] = { pos3[3 * j] - pos3[3 * i], pos3[3 * j + 1] - pos3[3 * i + 1], pos3[3 * j + 2] - pos3[3 * i + 2] };
                double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                double w;
                if (law == 0) w = G * mass[i] * mass[j] / (std::sqrt(r2) * (r2 + S));
                else { double q = r2 + S; w = G * mass[i] * mass[j] / (q * std::sqrt(q)); }
                if (r2 == 0.0) w = 0.0;
                F[0] += w * d[0]; F[1] += w * d[1]; F[2] += w * d[2];
            }
            force3[3 * k] = F[0]; force3[3 * k + 1] = F[1]; force3[3 * k + 2] = F[2];
        }
    });
    return 0;
}

/* FP64 energy / momenta of a state (O(n^2) potential). */
int orc_fp64_diagnostics(const double* pos3, const double* vel3, const double* mass, size_t n, double G, double S,
                         int law, int nthreads, double* out11) {
    double eps = std::sqrt(S);
    std::vector<double> pe(n, 0.0);
    parallel_slices(n, nthreads, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double s = 0.0;
            for (size_t j = i + 1; j < n; ++j) {
                double d[3] = { pos3[3 * j] - pos3[3 * i], pos3[3 * j + 1] - pos3[3 * i + 1], pos3[3 * j + 2] - pos3[3 * i + 2] };
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                double phi = (law == 0) ? -(1.0 / eps) * (M_PI / 2 - std::atan(r / eps)) : -1.0 / std::sqrt(r * r + S);
                s += G * mass[i] * mass[j] * phi;
            }
            pe[i] = s;
        }
    });
    double K = 0, U = 0, p[3] = {0, 0, 0}, L[3] = {0, 0, 0}, M = 0, c[3] = {0, 0, 0};
    for (size_t i = 0; i < n; ++i) {
        const double* x = pos3 + 3 * i; const double* v = vel3 + 3 * i; double m = mass[i];
        K += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        U += pe[i];
        for (int k = 0; k < 3; ++k) { p[k] += m * v[k]; c[k] += m * x[k]; }
        L[0] += m * (x[1] * v[2] - x[2] * v[1]);
        L[1] += m * (x[2] * v[0] - x[0] * v[2]);
        L[2] += m * (x[0] * v[1] - x[1] * v[0]);
        M += m;
    }
    out11[0] = K; out11[1] = U; out11[2] = K + U;
    out11[3] = p[0]; out11[4] = p[1]; out11[5] = p[2];
    out11[6] = L[0]; out11[7] = L[1]; out11[8] = L[2];
    out11[9] = M; out11[10] = 0.0;
    return 0;
}

int orc_threads_default(void) {
    unsigned hc = std::thread::hardware_concurrency();
    int t = (int)(hc == 0 ? 8 : hc) - 1;
    return t < 1 ? 1 : (t > 31 ? 31 : t);
}

} /* extern "C" */
