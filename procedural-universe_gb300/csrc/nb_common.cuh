// nb_common.cuh -- device helpers shared by the N-body kernels (sm_103a).
//
// Float arithmetic that must round exactly like the reference's CPU code
// (octree keys, node bounds, centre of mass, opening test) goes through the
// explicit round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn) so that nvcc never contracts it into a fused multiply-add.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nb {

// Device-side error codes written to the handle's error word.
enum : int {
    DEV_OK = 0,
    DEV_WAIT_TIMEOUT = 1,      // a bounded mbarrier wait ran out
    DEV_STACK_OVERFLOW = 2,    // traversal stack exceeded its bound
    DEV_TREE_OVERFLOW = 3,     // more tree nodes than allocated
    DEV_BAD_INPUT = 4,         // NaN / inf found in the state
};

// Upper bound of polls of an mbarrier before a wait is abandoned. Each
// try_wait already suspends for a hardware time slice, so this is seconds.
constexpr uint32_t kMaxPolls = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared (TMA engine), completion signalled on bar.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: true when the phase completed, false when the poll budget ran
// out (a budget of 0 gives up at once).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t polls = kMaxPolls) {
    for (uint32_t i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Hardware approximate reciprocal square root (MUFU.RSQ), flush-to-zero.
// atomicAdd with acquire-release semantics at GPU scope: the caller's earlier
// writes are visible to whoever later acquires this location, and the
// caller sees the writes released to it by earlier adders (the bottom-up
// tree passes: the last child to arrive reads its siblings' results).
__device__ __forceinline__ int atomic_add_acq_rel(int* p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Kahan accumulation of x into (s, c); the represented value is s - c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

__device__ __forceinline__ void record_error(int* err, int code) {
    if (err) atomicCAS(err, 0, code);
}

}  // namespace nb
