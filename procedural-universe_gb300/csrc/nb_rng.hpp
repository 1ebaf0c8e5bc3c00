// nb_rng.hpp -- counter-based random numbers shared by host and device code.
//
// splitmix64 (Steele, Lea, Flood 2014) turns a 64-bit seed into a key;
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11, "Parallel random
// numbers: as easy as 1, 2, 3") maps (counter, key) to four 32-bit words.
// Every body draws from its own counter stream (body index, draw number), so
// a body's initial conditions depend only on (seed, index) and are identical
// whatever thread or device generates them.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define NB_HD __host__ __device__ __forceinline__
#else
#define NB_HD inline
#endif

namespace nb {

NB_HD uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

NB_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

struct Philox4 {
    uint32_t v[4];
};

// Philox-4x32 with 10 rounds (published constants of the paper).
NB_HD Philox4 philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, c0, hi0, lo0);
        mulhilo32(M1, c2, hi1, lo1);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += W0; k1 += W1;
    }
    Philox4 o;
    o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
    return o;
}

// Stream of uniforms in (0, 1) (53-bit, never 0 or 1) for one body.
struct BodyRng {
    uint32_t k0, k1, body, stream;
    uint32_t ctr = 0;
    Philox4 buf{};
    int left = 0;
    NB_HD BodyRng(uint64_t seed, uint64_t body_index, uint32_t stream_id) {
        const uint64_t key = splitmix64(seed);
        k0 = (uint32_t)key;
        k1 = (uint32_t)(key >> 32);
        body = (uint32_t)body_index;
        stream = stream_id ^ (uint32_t)(body_index >> 32);
    }
    NB_HD uint32_t next32() {
        if (left == 0) {
            buf = philox4x32(body, ctr++, stream, 0x6E626F64u, k0, k1);
            left = 4;
        }
        return buf.v[--left];
    }
    NB_HD double uniform() {
        const uint64_t a = next32(), b = next32();
        const uint64_t bits = (a << 21) ^ (b >> 11);   // 53 bits
        return ((double)bits + 0.5) * (1.0 / 9007199254740992.0);
    }
};

}  // namespace nb
