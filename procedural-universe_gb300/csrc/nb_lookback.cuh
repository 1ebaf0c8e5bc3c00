// nb_lookback.cuh -- single-pass prefix sums across thread blocks by decoupled
// look-back (Merrill and Garland, "Single-pass Parallel Prefix Scan with
// Decoupled Look-back", NVIDIA technical report NVR-2016-002).
//
// A tile takes its index from an atomic counter in the order blocks start, so
// it only ever waits for tiles that started before it.  It publishes its own
// total (flag 1) at once, then walks back over its predecessors adding their
// totals until one has published an inclusive prefix (flag 2), and publishes
// its own inclusive prefix.  A status word is (flag << 32) | value in one
// 64-bit word, so relaxed loads and stores at GPU scope suffice (no other
// data travels with it) and the loads of a window can overlap.  Every wait is
// bounded: a tile that gives up reports DEV_WAIT_TIMEOUT through the error
// word and carries on with what it has summed (the step is reported failed).
#pragma once
#include <cstdint>
#include "nb_common.cuh"
#include "nb_scan.cuh"

namespace nb {

constexpr uint32_t kLookbackPolls = 1u << 20;   // x >= 64 ns of back-off: >= 60 ms per wait

__device__ __forceinline__ void lb_publish(unsigned long long* p, uint32_t flag, uint32_t value) {
    const unsigned long long w = ((unsigned long long)flag << 32) | (unsigned long long)value;
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(w) : "memory");
}

__device__ __forceinline__ unsigned long long lb_load(const unsigned long long* p) {
    unsigned long long w;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(p) : "memory");
    return w;
}

// Exclusive prefix of tile `tile` from the status words status[j * stride]
// of tiles j < tile, read by one thread kLbWindow predecessors at a time (the
// loads of a window are independent and in flight together, so a walk back
// over many tiles costs 1/kLbWindow of the round trips).
constexpr int kLbWindow = 4;

__device__ __forceinline__ uint32_t lb_exclusive(const unsigned long long* status, int tile, int stride, int* err) {
    uint32_t sum = 0;
    int j = tile - 1;
    uint32_t polls = 0;
    while (j >= 0) {
        unsigned long long w[kLbWindow];
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k)
            w[k] = (j - k >= 0) ? lb_load(status + (size_t)(j - k) * (size_t)stride) : (2ull << 32);
        // take the window up to its first inclusive prefix; a gap before it means waiting
        uint32_t part = 0;
        bool done = false, gap = false;
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k) {
            if (done || gap) continue;
            const uint32_t flag = (uint32_t)(w[k] >> 32);
            if (flag == 0u) { gap = true; continue; }
            part += (uint32_t)w[k];
            if (flag == 2u) done = true;
        }
        if (gap) {
            if (++polls > kLookbackPolls) {
                record_error(err, DEV_WAIT_TIMEOUT);
                return sum;
            }
            __nanosleep(64);
            continue;   // the same window again
        }
        sum += part;
        if (done) break;
        j -= kLbWindow;
    }
    return sum;
}

// The same for the first warp of a block, 32 predecessors per round (one per
// lane); every lane returns the prefix.
__device__ __forceinline__ uint32_t lb_exclusive_warp(const unsigned long long* status, int tile, int* err) {
    const int lane = threadIdx.x & 31;
    uint32_t sum = 0;
    int base = tile - 1;
    uint32_t polls = 0;
    while (base >= 0) {
        const int j = base - lane;
        const unsigned long long w = j >= 0 ? lb_load(status + j) : (2ull << 32);   // before tile 0: prefix 0
        const uint32_t flag = (uint32_t)(w >> 32);
        const unsigned incl = __ballot_sync(0xffffffffu, flag == 2u);
        const unsigned empty = __ballot_sync(0xffffffffu, flag == 0u);
        const int first = incl ? __ffs(incl) - 1 : 31;
        const unsigned upto = first == 31 ? 0xffffffffu : ((2u << first) - 1u);
        if (empty & upto) {
            if (++polls > kLookbackPolls) {
                if (lane == 0) record_error(err, DEV_WAIT_TIMEOUT);
                return sum;
            }
            __nanosleep(64);
            continue;
        }
        uint32_t v = lane <= first ? (uint32_t)w : 0u;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        sum += v;
        if (incl) break;
        base -= 32;
    }
    return sum;
}

// The tile index of this block: blocks take consecutive indices in the order
// they start.  Call with every thread of the block; returns the index.
__device__ __forceinline__ int lb_tile_index(int* ctr, int* sh) {
    if (threadIdx.x == 0) *sh = atomicAdd(ctr, 1);
    __syncthreads();
    const int t = *sh;
    __syncthreads();
    return t;
}

// Exclusive block-and-grid prefix of one value per thread of a tile: block
// scan (nb_scan.cuh's block_excl_scan), then the tile's offset by look-back on
// status[tile].  *grand (when non-null) receives the total of all tiles from
// the last tile.  sh_warp: 33 ints of shared memory; sh_off: one int.
__device__ __forceinline__ int lb_scan_tile(int v, int tile, int ntiles, unsigned long long* status, int* grand,
                                            int* sh_warp, int* sh_off, int* err) {
    int total;
    const int r = block_excl_scan(v, sh_warp, &total);
    if (threadIdx.x < 32) {
        uint32_t excl = 0;
        if (tile == 0) {
            if (threadIdx.x == 0) lb_publish(status, 2u, (uint32_t)total);
        } else {
            if (threadIdx.x == 0) lb_publish(status + tile, 1u, (uint32_t)total);
            excl = lb_exclusive_warp(status, tile, err);
            if (threadIdx.x == 0) lb_publish(status + tile, 2u, excl + (uint32_t)total);
        }
        if (threadIdx.x == 0) {
            if (grand && tile == ntiles - 1) *grand = (int)(excl + (uint32_t)total);
            *sh_off = (int)excl;
        }
    }
    __syncthreads();
    const int off = *sh_off;
    __syncthreads();
    return r + off;
}

}  // namespace nb
