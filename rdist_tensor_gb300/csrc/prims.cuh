// Device-wide primitives: exclusive scans and a stable LSD radix sort.
#pragma once
#include "common.cuh"

namespace exafac {

constexpr int kScanTile = 4096;  // elements per block in the scans

// Bytes of scratch the scans need for n elements.
inline size_t scan_scratch_bytes(int64_t n) { return sizeof(double) * (size_t)(ceil_div(n, kScanTile) + 2); }

// out[i] = sum_{j<i} in[i]; *total (device) = sum of all (may be null).
// Sums are formed blockwise (not in sequential order).
int scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total, void* scratch, cudaStream_t s);
int scan_exclusive_u32_to_i64(const uint32_t* in, int64_t* out, int64_t n, int64_t* total, void* scratch,
                              cudaStream_t s, int64_t* accum = nullptr);

// Inclusive scan of doubles.
int scan_inclusive_f64(const double* in, double* out, int64_t n, double* total, void* scratch, cudaStream_t s);

// Discrete CDF of nonnegative weights: out_i = S_i / S_{n-1} with S the
// blockwise inclusive scan, out_{n-1} = 1; *total (device) = S_{n-1}.
// gather (optional): weight i is in[gather[i]]; n_dev (optional): the length
// is min(n, *n_dev), n only sizes the launch.
int scan_cdf_f64(const double* in, double* out, int64_t n, double* total, void* scratch, cudaStream_t s,
                 const uint32_t* gather = nullptr, const int64_t* n_dev = nullptr);

// Stable LSD radix sort of `count` keys (kw = 1: 64-bit keys in lo; kw = 2:
// 128-bit (lo, hi)) over their low `bits` bits, carrying a uint32 payload.
// Results land in (lo_out, hi_out, pay_out); the *_tmp arrays are ping-pong
// buffers of the same sizes.  Scratch: radix_scratch_bytes(count).
size_t radix_scratch_bytes(int64_t count);
int radix_sort_pairs(int64_t count, int bits, int kw, const uint64_t* lo_in, const uint64_t* hi_in,
                     const uint32_t* pay_in, uint64_t* lo_out, uint64_t* hi_out, uint32_t* pay_out, uint64_t* lo_tmp,
                     uint64_t* hi_tmp, uint32_t* pay_tmp, void* scratch, cudaStream_t s);

}  // namespace exafac
