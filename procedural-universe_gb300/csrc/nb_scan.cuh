// nb_scan.cuh -- device-wide exclusive prefix sum of int32 values.
//
// Three launches: per-block scan with the block totals written out, a scan
// of the block totals by one block, and the add-back.  An optional device
// flag skips all three (used by radix passes the sort plan marks trivial).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace nb {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive block scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ int block_excl_scan(int v, int* sh_warp, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int inc = warp_incl_scan(v);
    if (lane == 31) sh_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? sh_warp[lane] : 0;
        const int wi = warp_incl_scan(w);
        if (lane < nw) sh_warp[lane] = wi - w;
        if (lane == nw - 1) sh_warp[32] = wi;
    }
    __syncthreads();
    const int r = sh_warp[warp] + inc - v;
    *total = sh_warp[32];
    __syncthreads();
    return r;
}

__global__ void k_scan_tiles(const int* in, int* out, int n, int* __restrict__ block_sums,
                             const int* __restrict__ skip) {
    if (skip && *skip) return;
    __shared__ int sh[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        sum += v[k];
    }
    int total;
    int run = block_excl_scan(sum, sh, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// One block scans the block totals (any count, in chunks) and writes the grand total.
__global__ void k_scan_block_sums(int* __restrict__ block_sums, int nblocks, int* __restrict__ grand_total,
                                  const int* __restrict__ skip) {
    if (skip && *skip) return;
    __shared__ int sh[33];
    int carry = 0;
    for (int b0 = 0; b0 < nblocks; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = i < nblocks ? block_sums[i] : 0;
        int total;
        const int e = block_excl_scan(v, sh, &total);
        if (i < nblocks) block_sums[i] = e + carry;
        carry += total;
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ block_sums,
                           const int* __restrict__ skip) {
    if (skip && *skip) return;
    const int add = block_sums[blockIdx.x];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) out[base + k] += add;
}

inline int scan_blocks(int n) { return (n + kScanTile - 1) / kScanTile; }

// out[i] = sum of in[0..i-1]; *grand_total (device) = sum of all. in may equal out.
// block_sums needs scan_blocks(n) ints.
inline cudaError_t exclusive_scan(const int* in, int* out, int n, int* block_sums, int* grand_total, cudaStream_t st,
                                  const int* skip = nullptr) {
    const int nb = scan_blocks(n);
    if (n <= 0) return cudaSuccess;
    k_scan_tiles<<<nb, kScanThreads, 0, st>>>(in, out, n, block_sums, skip);
    k_scan_block_sums<<<1, kScanThreads, 0, st>>>(block_sums, nb, grand_total, skip);
    k_scan_add<<<nb, kScanThreads, 0, st>>>(out, n, block_sums, skip);
    return cudaGetLastError();
}

}  // namespace nb
