// nb_gen.cu -- synthetic galaxies generated on the device, straight into a
// batch's state arrays (the batched form's nb_batch_add_generated and the
// served form's job admission).
//
// The step before the N-body path in the reference is a seeder filling the
// particle vector on the host (src/Sim/GalaxySeeder.cpp:43-144); here a
// galaxy-generation job makes its initial conditions where they are used.
// Each body comes from nb_seed_body.hpp (the host generator's code) and its
// own Philox stream.  The centre-of-mass shift needs the whole galaxy, so the
// bodies are made twice: a first pass sums m, m x, m v per chunk of kChunk
// bodies (double, fixed order inside a block), one thread per galaxy adds its
// chunks in order, and a second pass makes the bodies again, shifts them and
// rounds to float.  Both passes and the sums are deterministic, so a galaxy
// comes out the same in every batch and on every run; it differs from the
// host generator only by the rounding of the device math functions and of
// the summation order of the centre of mass.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include "nb_seed_body.hpp"

#include <algorithm>
#include <vector>

namespace nb {

namespace {

constexpr int kChunk = 2048;         // bodies per block of both passes
constexpr int kGenThreads = 256;

struct GenGal {
    uint64_t seed;
    long long off;    // first body in the batch arrays
    int n, model;
    double rel_x, rel_v[2];   // collision model: separation and relative velocity (radial, tangential)
};

__device__ __forceinline__ float gen_body(const GenGal& g, size_t i, double x[3], double v[3]) {
    using namespace seedbody;
    if (g.model == 1) {   // Plummer sphere, M = 1, a = 1 (nb_seed_plummer's defaults)
        BodyRng r(g.seed, i, kStreamPlummer);
        plummer_body(r, 1.0, 1.0, x, v);
        return (float)(1.0 / (double)g.n);
    }
    if (g.model == 2) {   // two Plummer spheres on a parabolic orbit (nb_seed_collision's defaults)
        const size_t h = (size_t)g.n / 2;
        const bool second = i >= h;
        const size_t cnt = second ? (size_t)g.n - h : h;
        BodyRng r(g.seed, i, kStreamCollision);
        plummer_body(r, 1.0, 1.0, x, v);
        const double sgn = second ? 0.5 : -0.5;
        x[0] += sgn * g.rel_x;
        v[0] += sgn * g.rel_v[0];
        v[1] += sgn * g.rel_v[1];
        return (float)(1.0 / (double)cnt);
    }
    // exponential disk + 10% Hernquist bulge (nb_seed_disk's defaults)
    const DiskParams p = disk_params((size_t)g.n, 1.0, 1.0, 0.1, 0.1, 0.2, 0.05);
    BodyRng r(g.seed, i, kStreamDisk);
    return disk_body(r, i, p, x, v);
}

// Pass 1: per chunk (galaxy, first body, count), sums of m, m x, m v.
__global__ void __launch_bounds__(kGenThreads) k_gen_sums(const GenGal* __restrict__ gals,
                                                          const int4* __restrict__ chunks, double* __restrict__ part) {
    __shared__ double red[7][kGenThreads];
    const int4 c = chunks[blockIdx.x];
    const GenGal g = gals[c.x];
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int k = threadIdx.x; k < c.z; k += kGenThreads) {
        double x[3], v[3];
        const double m = gen_body(g, (size_t)(c.y + k), x, v);
        s[0] += m;
        for (int a = 0; a < 3; ++a) { s[1 + a] += m * x[a]; s[4 + a] += m * v[a]; }
    }
    for (int q = 0; q < 7; ++q) red[q][threadIdx.x] = s[q];
    __syncthreads();
    for (int w = kGenThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int q = 0; q < 7; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 7) part[7 * (size_t)blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

// Per galaxy: add its chunks in order; centre of mass and its velocity.
__global__ void k_gen_centre(const int2* __restrict__ gal_chunks, int ngal, const double* __restrict__ part,
                             double* __restrict__ com) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngal) return;
    const int2 r = gal_chunks[g];   // first chunk, chunks
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < r.y; ++k)
        for (int q = 0; q < 7; ++q) s[q] += part[7 * (size_t)(r.x + k) + q];
    for (int q = 0; q < 6; ++q) com[6 * (size_t)g + q] = s[0] > 0 ? s[1 + q] / s[0] : 0.0;
}

// Pass 2: the bodies again, in the centre-of-mass frame, rounded to float.
__global__ void __launch_bounds__(kGenThreads) k_gen_write(const GenGal* __restrict__ gals,
                                                           const int4* __restrict__ chunks,
                                                           const double* __restrict__ com, float4* __restrict__ pos,
                                                           float4* __restrict__ vel) {
    const int4 c = chunks[blockIdx.x];
    const GenGal g = gals[c.x];
    const double* cm = com + 6 * (size_t)c.x;
    for (int k = threadIdx.x; k < c.z; k += kGenThreads) {
        double x[3], v[3];
        const size_t i = (size_t)(c.y + k);
        const float m = gen_body(g, i, x, v);
        pos[g.off + (long long)i] = make_float4((float)(x[0] - cm[0]), (float)(x[1] - cm[1]), (float)(x[2] - cm[2]), m);
        vel[g.off + (long long)i] = make_float4((float)(v[0] - cm[3]), (float)(v[1] - cm[4]), (float)(v[2] - cm[5]), 0.f);
    }
}

template <typename T>
cudaError_t upload_async(T** d, const std::vector<T>& h, cudaStream_t st) {
    cudaError_t e = dev_alloc(d, std::max<size_t>(1, h.size()) * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

}  // namespace

// Generates every listed galaxy into pos / vel (position compensation and
// velocity compensation stay as they are: zero in a freshly reserved batch).
// Waits for the stream before it returns (its tables are freed).
cudaError_t gen_galaxies(const std::vector<GenSpec>& specs, float4* pos, float4* vel, cudaStream_t st) {
    if (specs.empty()) return cudaSuccess;
    std::vector<GenGal> gals(specs.size());
    std::vector<int4> chunks;
    std::vector<int2> gal_chunks(specs.size());
    for (size_t k = 0; k < specs.size(); ++k) {
        const GenSpec& s = specs[k];
        GenGal& g = gals[k];
        g.seed = s.seed;
        g.off = (long long)s.off;
        g.n = (int)s.n;
        g.model = s.model;
        g.rel_x = g.rel_v[0] = g.rel_v[1] = 0.0;
        if (s.model == 2) {   // nb_seed_collision: separation 10, pericentre 1, total mass 2, G = 1
            const double sep = 10.0, peri = 1.0, Mt = 2.0;
            const double vrel = std::sqrt(2.0 * Mt / sep);
            const double vt = std::sqrt(2.0 * Mt * peri) / sep;
            g.rel_x = sep;
            g.rel_v[0] = -std::sqrt(std::max(0.0, vrel * vrel - vt * vt));
            g.rel_v[1] = vt;
        }
        gal_chunks[k] = make_int2((int)chunks.size(), (int)((s.n + kChunk - 1) / kChunk));
        for (size_t b = 0; b < s.n; b += kChunk)
            chunks.push_back(make_int4((int)k, (int)b, (int)std::min<size_t>(kChunk, s.n - b), 0));
    }
    GenGal* d_gals = nullptr;
    int4* d_chunks = nullptr;
    int2* d_gal_chunks = nullptr;
    double *d_part = nullptr, *d_com = nullptr;
    cudaError_t e = upload_async(&d_gals, gals, st);
    if (e == cudaSuccess) e = upload_async(&d_chunks, chunks, st);
    if (e == cudaSuccess) e = upload_async(&d_gal_chunks, gal_chunks, st);
    if (e == cudaSuccess) e = dev_alloc(&d_part, 7 * chunks.size() * sizeof(double));
    if (e == cudaSuccess) e = dev_alloc(&d_com, 6 * gals.size() * sizeof(double));
    if (e == cudaSuccess) {
        k_gen_sums<<<(unsigned)chunks.size(), kGenThreads, 0, st>>>(d_gals, d_chunks, d_part);
        k_gen_centre<<<(unsigned)((gals.size() + 127) / 128), 128, 0, st>>>(d_gal_chunks, (int)gals.size(), d_part,
                                                                           d_com);
        k_gen_write<<<(unsigned)chunks.size(), kGenThreads, 0, st>>>(d_gals, d_chunks, d_com, pos, vel);
        e = cudaGetLastError();
    }
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    for (void* p : {(void*)d_gals, (void*)d_chunks, (void*)d_gal_chunks, (void*)d_part, (void*)d_com}) dev_free(p, st);
    return e;
}

}  // namespace nb
