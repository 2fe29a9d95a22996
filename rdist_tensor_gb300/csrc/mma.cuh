// Warp-level tensor-core helpers: mma.sync m16n8k8 with TF32 operands and
// FP32 accumulation, and the TF32 rounding of FP32 values.
#pragma once

#include "common.cuh"

namespace exafac {

// TF32 rounding (10 mantissa bits), to nearest with ties away from zero, in
// integer arithmetic: adding half a TF32 ulp (bit 12) to the sign-magnitude
// pattern and clearing the 13 dropped bits rounds the magnitude; a carry moves
// the exponent up (to infinity past the largest TF32 value).  Infinities and
// NaNs pass through.  Same results as cvt.rna.tf32.f32, without the
// conversion unit.
__device__ __forceinline__ float round_tf32(float x) {
    const uint32_t b = __float_as_uint(x);
    if ((b & 0x7f800000u) == 0x7f800000u) return x;
    return __uint_as_float((b + 0x1000u) & 0xffffe000u);
}

// D += A B for one 16 x 8 x 8 block: a = A fragment (rows gid, gid + 8;
// columns tig, tig + 4), b = B fragment (rows tig, tig + 4; column gid),
// c = rows gid, gid + 8 x columns 2 tig, 2 tig + 1 (gid = lane / 4,
// tig = lane % 4).
__device__ __forceinline__ void mma_tf32_16x8x8(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// x = hi + lo with hi = TF32(x) and lo = x - hi exact in FP32 (the tensor
// cores read lo's top 10 mantissa bits): the operands of a 3xTF32 product
// hi*hi + hi*lo + lo*hi, accurate to about 2^-21 relative.
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
    const float h = round_tf32(x);
    hi = __float_as_uint(h);
    lo = __float_as_uint(x - h);
}

}  // namespace exafac
