// Bulk asynchronous copies global -> shared (the copy engine's 1-D form,
// cp.async.bulk) completed on an mbarrier, for kernels that stream
// contiguous tiles and want the next tile in flight while they work on the
// current one.  Addresses and sizes of a copy must be multiples of 16 bytes.
#pragma once

#include "common.cuh"

namespace exafac {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Orders this thread's earlier shared-memory accesses (generic proxy) before
// later bulk copies into the same memory (async proxy); also publishes
// mbarrier initialisation to the copy engine.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// The single arrival of a phase, announcing the bytes its copies will bring.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// One poll of the phase of parity `phase`: true once it has completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return done != 0;
}

// Asynchronous copies global -> shared of 16 or 4 bytes per thread (the
// Ampere-style cp.async): src_bytes < size zero-fills the rest (0: no read).
// Completion per thread by commit groups.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// An arrival on *bar once this thread's earlier cp.async copies have landed
// (the barrier's count must include it: no pending-count increment).
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// All but the `N` most recent groups of this thread complete.
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of parity `phase`: at most `polls` polls and at most
// about one second (each try_wait may suspend for a hardware-chosen time, so
// the poll count alone does not bound the wait).  False when it ran out.
__device__ __forceinline__ bool mbar_wait_limited(uint64_t* bar, uint32_t phase, uint32_t polls) {
    const uint64_t deadline = global_ns() + 1000000000ull;
    for (uint32_t it = 0; it < polls; it++) {
        if (mbar_try_wait(bar, phase)) return true;
        if ((it & 255u) == 255u && global_ns() > deadline) return false;
    }
    return false;
}

// Waits for the phase of parity `phase` to complete, at most kBulkWaitPolls
// polls (each try_wait may itself suspend briefly).  False on timeout.
constexpr uint32_t kBulkWaitPolls = 1u << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    for (uint32_t it = 0; it < kBulkWaitPolls; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

}  // namespace exafac
