// Carry fix-up of the chunked segmented reductions over row-sorted hits
// (sort_lookup.hpp:347-371 computes the same row sums serially): rows that
// cross a chunk border are summed from the chunks' carries in chunk order.
#pragma once
#include "engine.cuh"

namespace exafac {

constexpr uint32_t kNoRow = 0xffffffffu;  // rows are < 2^32 - 1

// Crossing rows, one warp per chunk c0 whose last row continues: the row's
// carries carry_last[c0] + sum over c in (c0, c1] of carry_first[c], c1 the
// last chunk that starts inside the row: the chunk of the row's last hit,
// seg_start[carry_seg[c0] + 1] - 1, when the run starts are given (one load
// however long the row); otherwise the chunks that do form a prefix of c0+1,
// c0+2, ..., found 32 at a time by ballot.  Spans of up to 32 chunks
// (almost every row): lane = column, chunks summed in order.  Longer spans
// (the hot rows): lane l sums chunks c0+1+l, c0+1+l+32, ... over all 32 padded
// columns, then a butterfly reduce-scatter leaves column l's total in lane l.
// Both orders are fixed, so results are reproducible run to run.
// carry_seg != null: Mc is compact and the row's output index is carry_seg[c0].
template <typename TA, int kChunk, int CB = 1>  // CB column blocks of 32 (carry stride 32 CB)
__global__ void __launch_bounds__(256) segfix_kernel(int R, int ldm, const int64_t* __restrict__ counters, int64_t cap,
                                                     const uint32_t* __restrict__ carry_row,
                                                     const uint32_t* __restrict__ carry_seg,
                                                     const int64_t* __restrict__ seg_start,
                                                     const uint32_t* __restrict__ keys,
                                                     const TA* __restrict__ carry_first,
                                                     const TA* __restrict__ carry_last, TA* __restrict__ Mc) {
    pdl_wait();
    pdl_trigger();
    const int64_t H = min(counters[1], cap);
    const int64_t nchunks = (H + kChunk - 1) / kChunk;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned full = 0xffffffffu;
    for (int64_t c0 = warp; c0 < nchunks; c0 += nwarps) {
        const uint32_t row = carry_row[c0];
        if (row == kNoRow) continue;
        const int64_t out = carry_seg ? (int64_t)carry_seg[c0] : (int64_t)row;
        int64_t c1 = c0;
        if (seg_start) {
            c1 = (min(seg_start[out + 1], H) - 1) / kChunk;
        } else {
            for (int64_t b = c0 + 1;; b += 32) {
                const int64_t m = b + lane;
                const bool on = m < nchunks && keys[m * kChunk] == row;
                const unsigned bal = __ballot_sync(full, on);
                c1 = b + __popc(bal) - 1;
                if (bal != full) break;
            }
        }
        // Columns R .. ldm - 1 of a padded FP32 row are written as zeros: the
        // solve reads whole rows, and the row's memory holds whatever the
        // workspace held before (a NaN there would survive the product with
        // Phi's zero padding).
        if (c1 - c0 <= 32) {  // short span: column per lane, chunks in order
            for (int cb = 0; cb < CB; cb++) {
                const int col = 32 * cb + lane;
                if (col >= R) {
                    if (col < ldm) Mc[out * ldm + col] = TA(0);
                    continue;
                }
                TA v = carry_last[c0 * (32 * CB) + col];
#pragma unroll 4
                for (int64_t m = c0 + 1; m <= c1; m++) v += carry_first[m * (32 * CB) + col];
                Mc[out * ldm + col] = v;
            }
            continue;
        }
        for (int cb = 0; cb < CB; cb++) {
            TA acc[32];
#pragma unroll
            for (int k = 0; k < 32; k++) acc[k] = 0;
            for (int64_t m = c0 + 1 + lane; m <= c1; m += 32) {
                const TA* src = carry_first + m * (32 * CB) + 32 * cb;
#pragma unroll
                for (int k = 0; k < 32; k++) acc[k] += src[k];
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) {
                const bool upper = (lane & off) != 0;
#pragma unroll
                for (int k = 0; k < off; k++) {
                    const TA send = upper ? acc[k] : acc[k + off];
                    const TA keep = upper ? acc[k + off] : acc[k];
                    acc[k] = keep + __shfl_xor_sync(full, send, off);
                }
            }
            const int col = 32 * cb + lane;
            if (col < R) Mc[out * ldm + col] = carry_last[c0 * (32 * CB) + col] + acc[0];
            else if (col < ldm) Mc[out * ldm + col] = TA(0);
        }
    }
}

}  // namespace exafac
