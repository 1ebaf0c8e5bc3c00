// nb_fp64.cu -- FP64 direct-sum oracle (K8) and FP64 diagnostics.
//
// The FP64 oracle measures force error: for m sampled target bodies it
// sums the exact force law in double precision over all n sources, from the
// same float positions and masses the FP32 kernels use.  The diagnostics
// reduce kinetic energy, linear and angular momentum, mass and centre of mass
// in FP64; the O(n^2) potential evaluates each pair term in FP32 and
// accumulates it in FP64.  All reductions write per-block partials that one
// block folds in a fixed order, so results are deterministic.
#include "nb_common.cuh"
#include "nb_internal.hpp"

namespace nb {

constexpr int kF64Block = 256;
constexpr int kF64Targets = 8;

template <int LAW>
__global__ void __launch_bounds__(kF64Block) k_fp64_forces(const float4* __restrict__ pos, int n,
                                                            const int32_t* __restrict__ targets, int m, double S,
                                                            double G, double* __restrict__ out3) {
    __shared__ double red[kF64Targets][3][kF64Block / 32];
    const int t0 = blockIdx.x * kF64Targets;
    double xi[kF64Targets], yi[kF64Targets], zi[kF64Targets];
    int ii[kF64Targets];
    double fx[kF64Targets], fy[kF64Targets], fz[kF64Targets];
#pragma unroll
    for (int k = 0; k < kF64Targets; ++k) {
        const int t = min(t0 + k, m - 1);
        ii[k] = targets[t];
        const float4 p = pos[ii[k]];
        xi[k] = p.x; yi[k] = p.y; zi[k] = p.z;
        fx[k] = fy[k] = fz[k] = 0.0;
    }
    for (int j = threadIdx.x; j < n; j += kF64Block) {
        const float4 pj = pos[j];
#pragma unroll
        for (int k = 0; k < kF64Targets; ++k) {
            const double dx = (double)pj.x - xi[k], dy = (double)pj.y - yi[k], dz = (double)pj.z - zi[k];
            const double r2 = dx * dx + dy * dy + dz * dz;
            double w;
            if (LAW == NB_LAW_REFERENCE) w = (double)pj.w / (sqrt(r2) * (r2 + S));
            else { const double q = r2 + S; w = (double)pj.w / (q * sqrt(q)); }
            if (j == ii[k] || r2 == 0.0) w = 0.0;
            fx[k] += w * dx; fy[k] += w * dy; fz[k] += w * dz;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kF64Targets; ++k) {
        double a = fx[k], b = fy[k], c = fz[k];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
        }
        if (lane == 0) { red[k][0][warp] = a; red[k][1][warp] = b; red[k][2][warp] = c; }
    }
    __syncthreads();
    if (threadIdx.x < kF64Targets * 3) {
        const int k = threadIdx.x / 3, c = threadIdx.x % 3;
        if (t0 + k < m) {
            double s = 0.0;
            for (int w = 0; w < kF64Block / 32; ++w) s += red[k][c][w];
            const float mi = pos[ii[k]].w;
            out3[(size_t)(t0 + k) * 3 + c] = G * (double)mi * s;
        }
    }
}

// Per-body FP64 terms: K, p, L, M, m*x, plus the pair potential sum of body
// i against every other body (FP32 terms, FP64 accumulation).
constexpr int kDiagTerms = 12;   // K px py pz Lx Ly Lz M mx my mz U

template <int LAW>
__global__ void __launch_bounds__(kF64Block) k_diag_partial(const float4* __restrict__ pos,
                                                             const float4* __restrict__ posc,
                                                             const float4* __restrict__ vel,
                                                             const float4* __restrict__ velc,
                                                             const float4* __restrict__ acc, float half_dt, int n,
                                                             int n_pad, float eps, float S, int with_potential,
                                                             double* __restrict__ partial) {
    __shared__ float4 tile[kF64Block];
    __shared__ double red[kDiagTerms][kF64Block / 32];
    const int i = blockIdx.x * kF64Block + threadIdx.x;
    const float4 pi = pos[i];   // i < n_pad always (grid covers n_pad exactly)
    double term[kDiagTerms];
#pragma unroll
    for (int k = 0; k < kDiagTerms; ++k) term[k] = 0.0;
    if (i < n) {
        const float4 xc = posc[i], v = vel[i], vc = velc[i];
        const double m = pi.w;
        const double x = (double)pi.x - xc.x, y = (double)pi.y - xc.y, z = (double)pi.z - xc.z;
        double vx = (double)v.x - vc.x, vy = (double)v.y - vc.y, vz = (double)v.z - vc.z;
        if (acc) {
            const float4 a = acc[i];
            vx += (double)a.x * half_dt; vy += (double)a.y * half_dt; vz += (double)a.z * half_dt;
        }
        term[0] = 0.5 * m * (vx * vx + vy * vy + vz * vz);
        term[1] = m * vx; term[2] = m * vy; term[3] = m * vz;
        term[4] = m * (y * vz - z * vy);
        term[5] = m * (z * vx - x * vz);
        term[6] = m * (x * vy - y * vx);
        term[7] = m;
        term[8] = m * x; term[9] = m * y; term[10] = m * z;
    }
    if (with_potential) {
        double u = 0.0;
        for (int j0 = 0; j0 < n_pad; j0 += kF64Block) {
            __syncthreads();
            tile[threadIdx.x] = pos[j0 + threadIdx.x];
            __syncthreads();
            float s = 0.f;
            for (int jj = 0; jj < kF64Block; ++jj) {
                const float4 pj = tile[jj];
                const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                float t;
                if (LAW == NB_LAW_REFERENCE) t = pj.w * atanf(eps * rsqrtf(r2));   // (pi/2 - atan(r/eps))
                else t = pj.w * rsqrtf(r2 + S);
                s += (j0 + jj == i) ? 0.f : t;
            }
            u += (double)s;
        }
        // each pair counted twice
        term[11] = (LAW == NB_LAW_REFERENCE) ? -0.5 * (double)pi.w * u / (double)eps : -0.5 * (double)pi.w * u;
        if (i >= n) term[11] = 0.0;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kDiagTerms; ++k) {
        double a = term[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) red[k][warp] = a;
    }
    __syncthreads();
    if (threadIdx.x < kDiagTerms) {
        double s = 0.0;
        for (int w = 0; w < kF64Block / 32; ++w) s += red[threadIdx.x][w];
        partial[(size_t)blockIdx.x * kDiagTerms + threadIdx.x] = s;
    }
}

__global__ void k_diag_final(const double* __restrict__ partial, int nblocks, double G, double* __restrict__ out) {
    __shared__ double red[kDiagTerms][32];
    const int k = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (k < kDiagTerms) {
        double s = 0.0;
        for (int b = lane; b < nblocks; b += 32) s += partial[(size_t)b * kDiagTerms + k];
        red[k][lane] = s;
    }
    __syncthreads();
    if (threadIdx.x < kDiagTerms) {
        double s = 0.0;
        for (int l = 0; l < 32; ++l) s += red[threadIdx.x][l];
        out[threadIdx.x] = (threadIdx.x == 11) ? G * s : s;
    }
}

cudaError_t fp64_forces(nb_sim* sim, const int32_t* d_targets, size_t m, double* d_out3) {
    if (m == 0) return cudaSuccess;
    const int blocks = (int)((m + kF64Targets - 1) / kF64Targets);
    if (sim->prm.law == NB_LAW_PLUMMER)
        k_fp64_forces<NB_LAW_PLUMMER><<<blocks, kF64Block, 0, sim->stream>>>(
            sim->pos, (int)sim->n, d_targets, (int)m, sim->prm.softening2, sim->prm.G, d_out3);
    else
        k_fp64_forces<NB_LAW_REFERENCE><<<blocks, kF64Block, 0, sim->stream>>>(
            sim->pos, (int)sim->n, d_targets, (int)m, sim->prm.softening2, sim->prm.G, d_out3);
    return cudaGetLastError();
}

// out: [K, px, py, pz, Lx, Ly, Lz, M, mx, my, mz, U]
cudaError_t fp64_diagnostics_ex(nb_sim* sim, float half_dt, bool with_acc, bool with_potential, double* d_out) {
    const int nblocks = (int)(sim->n_pad / kF64Block);
    const size_t need = (size_t)nblocks * kDiagTerms;
    if (need > sim->dscratch_cap) {
        dev_free(sim->dscratch, sim->stream);
        sim->dscratch = nullptr;
        sim->dscratch_cap = 0;
        cudaError_t e = dev_alloc(&sim->dscratch, need * sizeof(double));
        if (e != cudaSuccess) return e;
        sim->dscratch_cap = need;
    }
    const float eps = (float)sqrt(sim->prm.softening2);
    const float S = (float)sim->prm.softening2;
    const float4* acc = with_acc ? sim->acc : nullptr;
    if (sim->prm.law == NB_LAW_PLUMMER)
        k_diag_partial<NB_LAW_PLUMMER><<<nblocks, kF64Block, 0, sim->stream>>>(
            sim->pos, sim->posc, sim->vel, sim->velc, acc, half_dt, (int)sim->n, (int)sim->n_pad, eps, S,
            with_potential ? 1 : 0, sim->dscratch);
    else
        k_diag_partial<NB_LAW_REFERENCE><<<nblocks, kF64Block, 0, sim->stream>>>(
            sim->pos, sim->posc, sim->vel, sim->velc, acc, half_dt, (int)sim->n, (int)sim->n_pad, eps, S,
            with_potential ? 1 : 0, sim->dscratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diag_final<<<1, 32 * kDiagTerms, 0, sim->stream>>>(sim->dscratch, nblocks, sim->prm.G, d_out);
    return cudaGetLastError();
}

cudaError_t fp64_diagnostics(nb_sim* sim, double* d_out) { return fp64_diagnostics_ex(sim, 0.f, false, true, d_out); }

}  // namespace nb
