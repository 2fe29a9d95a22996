// Blackwell fifth-generation tensor-core primitives (tcgen05, sm_100a family):
// tensor-memory (TMEM) allocation, the single-CTA MMA reading both operands
// from shared memory through matrix descriptors and accumulating in FP32 in
// TMEM, its completion signalled on an mbarrier, and TMEM loads into
// registers.  Inline PTX; one thread issues the MMAs.
//
// Operand layout used here: K-major without swizzle.  A core matrix is 8 rows
// x 16 bytes (8 x 4 TF32 values), stored as 128 contiguous bytes; within a
// tile, core matrices adjacent along K are `lbo` bytes apart and 8-row groups
// `sbo` bytes apart:
//   byte(r, k) = (r / 8) * sbo + (k / 4) * lbo + (r % 8) * 16 + (k % 4) * 4.
#pragma once

#include "bulk.cuh"

namespace exafac {

// 64-bit shared-memory matrix descriptor: start address, leading (K) and
// stride (M/N) byte offsets in 16-byte units, descriptor version 1 (bits
// 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t umma_desc(const void* smem_ptr, uint32_t lbo, uint32_t sbo) {
    const uint32_t a = smem_u32(smem_ptr);
    uint64_t d = (uint64_t)((a & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// The same for the K-major 128-byte swizzled layout: 8-row atoms of 128-byte
// rows (1024 bytes, 1024-byte aligned), the 16-byte chunk c of row r stored
// at chunk c ^ (r % 8); 8-row groups 1024 bytes apart (stride offset), the
// leading offset unused (set to 16 bytes), swizzle mode 2 (bits 61-63).  A
// K step inside an atom advances the start address by its byte offset in the
// row.
__device__ __forceinline__ uint64_t umma_desc_sw128(const void* smem_ptr) {
    const uint32_t a = smem_u32(smem_ptr);
    uint64_t d = (uint64_t)((a & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;          // leading byte offset 16 (unused)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset 1024
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Byte offset of element (r, k) of a K-major, 128-byte swizzled operand whose
// K is cut into blocks of 32 FP32 values, `kb_bytes` apart (rows x 128 each).
__host__ __device__ __forceinline__ uint32_t sw128_off(int r, int k, uint32_t kb_bytes) {
    return (uint32_t)(k >> 5) * kb_bytes + (uint32_t)r * 128u + ((((uint32_t)k >> 2) & 7u) ^ ((uint32_t)r & 7u)) * 16u +
           ((uint32_t)k & 3u) * 4u;
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM allocation of `ncols` columns (a power of two, 32..512) by one whole
// warp; the base address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Ordering of tensor-core operations around thread barriers.
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D (TMEM, FP32) = A B^T (+ D when accumulate != 0); A: M x K, B: N x K, one
// K = 8 step of TF32.
__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// One arrival on *bar once every MMA this thread issued before has completed
// (their shared-memory reads included).
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of the warp's 32 TMEM lanes (lane = thread),
// starting at taddr (lane field in bits 16-31, column in bits 0-15).  The
// warp may only address the lane quarter 32 * (warp id % 4).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// The same for 16 columns.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Makes this thread's mbarrier initialisation visible to the other proxies
// (the tensor core's commit arrives on it).
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Round to TF32 (10 explicit mantissa bits), to nearest, ties away from zero.
__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

}  // namespace exafac
