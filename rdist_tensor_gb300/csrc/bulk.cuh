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
