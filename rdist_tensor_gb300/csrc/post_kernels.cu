// Sampled MTTKRP and post-processing, load-balanced (R <= 32 path), on the
// hits sorted by output row (hitsort.cu):
//
//   segred   M rows from fixed-size chunks of row-grouped hits: rows inside a
//            chunk are written directly, rows crossing a chunk border leave a
//            per-chunk carry (csr_based_spmm's row-chunked AXPYs,
//            sort_lookup.hpp:347-371, without atomics)
//   fixup    carries of each crossing row summed in chunk order
//   solve    U_r = M_r Phi (parallel_dsymm, accumulator_stationary.hpp:283-286),
//            thread per row over 32-row tiles, Gram partials of U in registers
//   normlev  u_r = U_r / sigma (renormalize_columns, distmat.hpp:85-138) and,
//            for CP-ARLS-LEV, l_r = u_r^T P u_r (compute_DAGAT, common.h:727-746)
#include "dense.cuh"
#include "engine.cuh"
#include "prims.cuh"

namespace exafac {

constexpr int kSegChunk = kSegChunkHits;  // hits per warp chunk in the segmented reduction

static int grid_capped(int64_t work, int threads, int64_t cap = 152 * 16) {
    int64_t b = ceil_div(work, threads);
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

// Segmented reduction over the row-sorted hits, lane = column (R <= 32).
// A warp takes a chunk of kSegChunk hits and stages them 32 at a time: each
// lane loads one hit (row, sample, value), a ballot marks where a new row
// starts, and every lane issues the group's 32 design-row loads before the
// first FMA, so the gathers overlap instead of forming one dependent chain
// per hit.  Mc[row] receives rows that lie inside one chunk; crossing rows
// leave carries (kCarryStride columns):
//   carry_first[c]: the chunk's first row when it started in an earlier chunk
//   carry_last[c]:  the chunk's last row when it continues in a later chunk,
//                   whose row goes to carry_row[c] (kNoRow when there is none)
constexpr uint32_t kNoRow = 0xffffffffu;  // rows are < 2^32 - 1

template <typename TD, typename TA>
__global__ void __launch_bounds__(256) segreduce_kernel(int R, const int64_t* __restrict__ counters, int64_t cap,
                                                        const uint32_t* __restrict__ keys,
                                                        const uint32_t* __restrict__ pay,
                                                        const uint32_t* __restrict__ ex_j,
                                                        const double* __restrict__ ex_val, const TD* __restrict__ D,
                                                        TA* __restrict__ Mc, TA* __restrict__ carry_first,
                                                        TA* __restrict__ carry_last, uint32_t* __restrict__ carry_row) {
    const int64_t H = min(counters[1], cap);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned full = 0xffffffffu;
    for (int64_t c = warp; c * kSegChunk < H; c += nwarps) {
        const int64_t cs = c * kSegChunk;
        const int64_t ce = min(H, cs + kSegChunk);
        uint32_t prev_row = kNoRow, next_row = kNoRow, first_row = kNoRow;
        if (lane == 0 && cs > 0) prev_row = keys[cs - 1];
        if (lane == 1 && ce < H) next_row = keys[ce];
        if (lane == 2) first_row = keys[cs];
        prev_row = __shfl_sync(full, prev_row, 0);
        next_row = __shfl_sync(full, next_row, 1);
        uint32_t cur = __shfl_sync(full, first_row, 2);  // row of the open segment
        bool first_seg = true;
        TA acc = 0;
        for (int64_t g = cs; g < ce; g += 32) {
            const int n = (int)min((int64_t)32, ce - g);
            uint32_t hj = 0, hr = kNoRow;
            TA hv = 0;
            if (lane < n) {
                hr = keys[g + lane];
                const uint32_t h = pay[g + lane];
                hj = ex_j[h];
                hv = (TA)ex_val[h];
            }
            uint32_t up = __shfl_up_sync(full, hr, 1);
            if (lane == 0) up = cur;
            const unsigned brk = __ballot_sync(full, lane < n && hr != up);
            TA d[32];
#pragma unroll
            for (int t = 0; t < 32; t++) {
                const uint32_t jt = __shfl_sync(full, hj, t);
                d[t] = (t < n && lane < R) ? (TA)D[(int64_t)jt * R + lane] : (TA)0;
            }
#pragma unroll
            for (int t = 0; t < 32; t++) {
                if (t < n) {
                    if ((brk >> t) & 1u) {  // the open segment ends inside the chunk
                        if (lane < R) {
                            if (first_seg && cur == prev_row) carry_first[c * kCarryStride + lane] = acc;
                            else Mc[(int64_t)cur * R + lane] = acc;
                        }
                        first_seg = false;
                        cur = __shfl_sync(full, hr, t);
                        acc = 0;
                    }
                    acc = fma(d[t], __shfl_sync(full, hv, t), acc);
                }
            }
        }
        const bool started_before = first_seg && cur == prev_row;
        const bool continues = cur == next_row;
        if (lane < R) {
            if (started_before) carry_first[c * kCarryStride + lane] = acc;
            else if (continues) carry_last[c * kCarryStride + lane] = acc;
            else Mc[(int64_t)cur * R + lane] = acc;
        }
        if (lane == 0) carry_row[c] = (!started_before && continues) ? cur : kNoRow;
    }
}

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
        if (c1 - c0 <= 32) {  // short span: column per lane, chunks in order
            for (int cb = 0; cb < CB; cb++) {
                const int col = 32 * cb + lane;
                if (col >= R) continue;
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
        }
    }
}

// Exact MTTKRP (execute_exact_mttkrp, sort_lookup.hpp:440-495) over the
// nonzeros sorted by their mode-n index: M[i_n] = sum of x * prod_{k != n}
// U_k[i_k] (mode order from 1.0), in the chunked segmented form of the
// sampled reduction, so the sums have a fixed order.  Lane l holds columns
// l + 32 b, b < CB; a lane loads one nonzero's value and coordinates per
// group of 32, and the factor rows of 8 nonzeros are gathered before their
// FMAs.  Carries use a stride of 32 CB doubles per chunk.
template <int CB>
__global__ void __launch_bounds__(256) exact_segreduce_kernel(int N, int n, int R, const int64_t* __restrict__ counters,
                                                              int64_t cap, const uint32_t* __restrict__ keys,
                                                              const uint32_t* __restrict__ pay,
                                                              const uint32_t* __restrict__ idx,
                                                              const double* __restrict__ vals, FactorPtrs f,
                                                              double* __restrict__ M, double* __restrict__ carry_first,
                                                              double* __restrict__ carry_last,
                                                              uint32_t* __restrict__ carry_row) {
    constexpr int ldc = 32 * CB;
    const int64_t H = min(counters[1], cap);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned full = 0xffffffffu;
    for (int64_t c = warp; c * kSegChunk < H; c += nwarps) {
        const int64_t cs = c * kSegChunk;
        const int64_t ce = min(H, cs + kSegChunk);
        uint32_t prev_row = kNoRow, next_row = kNoRow, first_row = kNoRow;
        if (lane == 0 && cs > 0) prev_row = keys[cs - 1];
        if (lane == 1 && ce < H) next_row = keys[ce];
        if (lane == 2) first_row = keys[cs];
        prev_row = __shfl_sync(full, prev_row, 0);
        next_row = __shfl_sync(full, next_row, 1);
        uint32_t cur = __shfl_sync(full, first_row, 2);
        bool first_seg = true;
        double acc[CB];
#pragma unroll
        for (int b = 0; b < CB; b++) acc[b] = 0.0;
        for (int64_t g = cs; g < ce; g += 32) {
            const int nn = (int)min((int64_t)32, ce - g);
            uint32_t hr = kNoRow, mi[kMaxModes];
            double hv = 0.0;
#pragma unroll
            for (int k = 0; k < kMaxModes; k++) mi[k] = 0;
            if (lane < nn) {
                hr = keys[g + lane];
                const uint32_t i = pay[g + lane];
                hv = vals[i];
#pragma unroll
                for (int k = 0; k < kMaxModes; k++)
                    if (k < N) mi[k] = idx[(int64_t)i * N + k];
            }
            uint32_t up = __shfl_up_sync(full, hr, 1);
            if (lane == 0) up = cur;
            const unsigned brk = __ballot_sync(full, lane < nn && hr != up);
            for (int t0 = 0; t0 < nn; t0 += 8) {
                double prod[8][CB];
#pragma unroll
                for (int u = 0; u < 8; u++) {
#pragma unroll
                    for (int b = 0; b < CB; b++) prod[u][b] = 1.0;
#pragma unroll
                    for (int k = 0; k < kMaxModes; k++) {
                        if (k < N && k != n) {
                            const int64_t row = __shfl_sync(full, mi[k], t0 + u);
#pragma unroll
                            for (int b = 0; b < CB; b++) {
                                const int col = lane + 32 * b;
                                if (col < R && t0 + u < nn) prod[u][b] *= f.U[k][row * R + col];
                            }
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int t = t0 + u;
                    if (t < nn) {
                        if ((brk >> t) & 1u) {
#pragma unroll
                            for (int b = 0; b < CB; b++) {
                                const int col = lane + 32 * b;
                                if (col < R) {
                                    if (first_seg && cur == prev_row) carry_first[c * ldc + col] = acc[b];
                                    else M[(int64_t)cur * R + col] = acc[b];
                                }
                                acc[b] = 0.0;
                            }
                            first_seg = false;
                            cur = __shfl_sync(full, hr, t);
                        }
                        const double v = __shfl_sync(full, hv, t);
#pragma unroll
                        for (int b = 0; b < CB; b++) acc[b] = fma(prod[u][b], v, acc[b]);
                    }
                }
            }
        }
        const bool started_before = first_seg && cur == prev_row;
        const bool continues = cur == next_row;
#pragma unroll
        for (int b = 0; b < CB; b++) {
            const int col = lane + 32 * b;
            if (col < R) {
                if (started_before) carry_first[c * ldc + col] = acc[b];
                else if (continues) carry_last[c * ldc + col] = acc[b];
                else M[(int64_t)cur * R + col] = acc[b];
            }
        }
        if (lane == 0) carry_row[c] = (!started_before && continues) ? cur : kNoRow;
    }
}

template <int CB>
static void launch_exact_mttkrp(Session& s, int n, double* M, FactorPtrs f, cudaStream_t st) {
    const int hb = 152 * 8;
    exact_segreduce_kernel<CB><<<hb, 256, 0, st>>>(s.N, n, s.R, s.counters, s.nnz, s.key_sorted, s.pay_sorted, s.idx,
                                                   s.vals, f, M, s.carry_first, s.carry_last, s.carry_row);
    count_launch();
    segfix_kernel<double, kSegChunk, CB><<<hb, 256, 0, st>>>(s.R, s.R, s.counters, s.nnz, s.carry_row, nullptr,
                                                             nullptr, s.key_sorted, s.carry_first, s.carry_last, M);
    count_launch();
}

int exact_mttkrp(Session& s, int n, double* M, cudaStream_t st) {
    EXAFAC_CUDA_TRY(cudaMemsetAsync(M, 0, sizeof(double) * s.dims[n] * s.R, st));
    EXAFAC_TRY(nonzeros_by_row(s, n, st));
    FactorPtrs f;
    for (int k = 0; k < kMaxModes; k++) f.U[k] = k < s.N ? s.F.U[k] : nullptr;
    const int cb = (s.R + 31) / 32;
    if (cb == 1) launch_exact_mttkrp<1>(s, n, M, f, st);
    else if (cb == 2) launch_exact_mttkrp<2>(s, n, M, f, st);
    else if (cb == 3) launch_exact_mttkrp<3>(s, n, M, f, st);
    else launch_exact_mttkrp<4>(s, n, M, f, st);
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// FP32 segmented reduction: four 8-lane groups per warp, each owning a chunk
// of kSegChunkF32 hits; within a group lane `sub` holds column block
// [4 sub, 4 sub + 4) of a float4 row (Q = f32_row_stride(R) / 4 blocks), so
// one 16-byte load brings a hit's four columns and the warp advances four
// hits per instruction.  Each lane loads four of its group's hits (row and
// the packed (sample, value) that travelled through the sort); hit t of the
// chunk is broadcast from lane t % 8 of the group.  Design rows are gathered 8 hits at a time before their FMAs.  Rows
// inside a chunk go straight to Mc (row stride 4Q floats); crossing rows
// leave the same carries as the FP64 form (kCarryStride floats per chunk).
template <int Q>
__global__ void __launch_bounds__(256) segreduce_f32_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                            const uint32_t* __restrict__ keys,
                                                            const uint64_t* __restrict__ pay64,
                                                            const uint32_t* __restrict__ chunk_seg,
                                                            const float4* __restrict__ D4, float4* __restrict__ Mc4,
                                                            float4* __restrict__ carry_first4,
                                                            float4* __restrict__ carry_last4,
                                                            uint32_t* __restrict__ carry_row,
                                                            uint32_t* __restrict__ carry_seg) {
    constexpr int C = kSegChunkF32;
    const int64_t H = min(counters[1], cap);
    const int64_t nchunks = (H + C - 1) / C;
    const int lane = threadIdx.x & 31, sub = lane & 7, grp = lane >> 3;
    const unsigned gmask = 0xffu << (8 * grp);
    const bool col = sub < Q;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t c = warp * 4 + grp; c < nchunks; c += nwarps * 4) {
        const int64_t cs = c * C;
        const int n = (int)min((int64_t)C, H - cs);
        const uint32_t prev_row = cs > 0 ? keys[cs - 1] : kNoRow;
        const uint32_t next_row = cs + n < H ? keys[cs + n] : kNoRow;
        uint32_t hr[4], hj[4];
        float hv[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {  // hit sub + 8 i of the chunk
            const int t = sub + 8 * i;
            hr[i] = kNoRow;
            hj[i] = 0;
            hv[i] = 0.f;
            if (t < n) {
                hr[i] = keys[cs + t];
                const uint64_t p = pay64[cs + t];
                hj[i] = (uint32_t)p;
                hv[i] = __uint_as_float((uint32_t)(p >> 32));
            }
        }
        uint32_t cur = __shfl_sync(gmask, hr[0], 0, 8);
        int64_t seg = chunk_seg[c];  // compact index of the run holding hit cs
        bool first_seg = true;
        float4 acc = zero4;
#pragma unroll
        for (int b = 0; b < C; b += 8) {
            float4 d[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const uint32_t jt = __shfl_sync(gmask, hj[b / 8], u, 8);
                d[u] = (b + u < n && col) ? D4[(int64_t)jt * Q + sub] : zero4;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int t = b + u;
                const uint32_t rt = __shfl_sync(gmask, hr[b / 8], u, 8);
                const float vt = __shfl_sync(gmask, hv[b / 8], u, 8);
                if (t < n) {
                    if (rt != cur) {  // the open segment ends inside the chunk
                        if (col) {
                            if (first_seg && cur == prev_row) carry_first4[c * 8 + sub] = acc;
                            else Mc4[seg * Q + sub] = acc;
                        }
                        first_seg = false;
                        cur = rt;
                        seg++;
                        acc = zero4;
                    }
                    acc.x = fmaf(d[u].x, vt, acc.x);
                    acc.y = fmaf(d[u].y, vt, acc.y);
                    acc.z = fmaf(d[u].z, vt, acc.z);
                    acc.w = fmaf(d[u].w, vt, acc.w);
                }
            }
        }
        const bool started_before = first_seg && cur == prev_row;
        const bool continues = cur == next_row;
        if (col) {
            if (started_before) carry_first4[c * 8 + sub] = acc;
            else if (continues) carry_last4[c * 8 + sub] = acc;
            else Mc4[seg * Q + sub] = acc;
        }
        if (sub == 0) {
            carry_row[c] = (!started_before && continues) ? cur : kNoRow;
            carry_seg[c] = (uint32_t)seg;
        }
    }
}

// U_r = M_r Phi for the touched rows, thread per row over 32-row tiles, and
// the packed Gram of these rows accumulated per lane (entries e = lane + 32q).
constexpr int kSolveWarps = 8;

template <typename TA, int Q>
size_t solve_gram_smem() {
    size_t tile = sizeof(TA) * kSolveWarps * 32 * 33;
    size_t red = sizeof(double) * kSolveWarps * 32 * Q;
    return sizeof(TA) * 32 * 32 + 2 * 544 + (tile > red ? tile : red);
}

template <typename TA, int Q>
__global__ void __launch_bounds__(kSolveWarps * 32) solve_gram_kernel(int R, const int64_t* __restrict__ counters,
                                                                   const uint32_t* __restrict__ touched,
                                                                   const TA* __restrict__ Mc,
                                                                   const double* __restrict__ Phi,
                                                                   double* __restrict__ U, double* __restrict__ part) {
    // Dynamic shared memory: phi[32*32] | pa[544] pb[544] | tile[warps][32][33]
    // (the per-warp Gram sums reuse the tile area at the end).
    extern __shared__ __align__(16) unsigned char smraw[];
    TA* phi = reinterpret_cast<TA*>(smraw);
    unsigned char* pa = smraw + sizeof(TA) * 32 * 32;
    unsigned char* pb = pa + 544;
    TA (*tile)[32][33] = reinterpret_cast<TA (*)[32][33]>(pb + 544);
    double (*red)[32 * Q] = reinterpret_cast<double (*)[32 * Q]>(pb + 544);
    const int P = R * (R + 1) / 2;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) phi[e] = (TA)Phi[e];
    for (int a = threadIdx.x; a < R; a += blockDim.x) {
        int base = a * R - a * (a - 1) / 2;
        for (int b = a; b < R; b++) {
            pa[base + b - a] = (unsigned char)a;
            pb[base + b - a] = (unsigned char)b;
        }
    }
    __syncthreads();
    double gacc[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) gacc[q] = 0.0;
    const int64_t nt = counters[2];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    TA (*ut)[33] = tile[w];
    for (int64_t base = warp * 32; base < nt; base += nwarps * 32) {
        const int64_t i = base + lane;
        TA m[32];
        if (i < nt) {
            const int64_t mrow = touched[i];
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < R) m[k] = Mc[mrow * R + k];
        }
        for (int cc = 0; cc < R; cc++) {
            TA acc = 0;
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < R) acc = fma(m[k], phi[k * R + cc], acc);
            ut[lane][cc] = (i < nt) ? acc : (TA)0;
        }
        __syncwarp();
        if (i < nt) {
            const int64_t row = touched[i];
            for (int cc = 0; cc < R; cc++) U[row * R + cc] = (double)ut[lane][cc];
        }
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int e = lane + 32 * q;
            if (e < P) {
                const int a = pa[e], b = pb[e];
                TA s = 0;
                for (int t = 0; t < 32; t++) s = fma(ut[t][a], ut[t][b], s);
                gacc[q] += (double)s;
            }
        }
        __syncwarp();
    }
    __syncthreads();  // the tile area becomes the reduction buffer
#pragma unroll
    for (int q = 0; q < Q; q++) red[w][lane + 32 * q] = gacc[q];
    __syncthreads();
    const int warps = blockDim.x >> 5;
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        double s = 0.0;
        for (int ww = 0; ww < warps; ww++) s += red[ww][e];
        part[(int64_t)blockIdx.x * P + e] = s;
    }
}

// u_r = U_r / sigma and, when P != null, l_r = u_r^T P u_r; thread per row
// over 32-row tiles staged in shared memory.
constexpr int kNormWarps = 4;

template <typename TA>
__global__ void __launch_bounds__(kNormWarps * 32) normlev_kernel(int R, const int64_t* __restrict__ counters,
                                                                 const uint32_t* __restrict__ touched,
                                                                 const double* __restrict__ sigma,
                                                                 const double* __restrict__ Pm,
                                                                 const int* __restrict__ degenerate,
                                                                 double* __restrict__ U, double* __restrict__ scores) {
    __shared__ TA psm[32 * 32];
    __shared__ double sg[32];
    __shared__ TA tile[kNormWarps][32][33];  // a warp's 32 rows, padded
    if (*degenerate) return;        // handled over all rows by scale_rows
    // P is symmetric: u^T P u = sum_a u_a (P_aa u_a + 2 sum_{b>a} P_ab u_b);
    // psm holds P_aa on the diagonal and 2 P_ab above it.
    for (int e = threadIdx.x; e < R * R; e += blockDim.x)
        if (Pm) psm[e] = (TA)((e / R == e % R) ? Pm[e] : 2.0 * Pm[e]);
    // Multiplying by 1/sigma differs from the reference's division by at
    // most one rounding.
    for (int c = threadIdx.x; c < R; c += blockDim.x) sg[c] = 1.0 / sigma[c];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    TA (*ut)[33] = tile[w];
    const int64_t nt = counters[2];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < nt; base += nwarps * 32) {
        const int64_t i = base + lane;
        if (i < nt) {
            const int64_t row = touched[i];
            for (int k = 0; k < R; k++) {
                const double v = U[row * R + k] * sg[k];
                U[row * R + k] = v;
                ut[lane][k] = (TA)v;
            }
        }
        __syncwarp();
        if (Pm && i < nt) {
            TA acc = 0;
            for (int a = 0; a < R; a++) {
                TA y = 0;
#pragma unroll 8
                for (int b = a; b < R; b++) y = fma(psm[a * R + b], ut[lane][b], y);
                acc = fma(ut[lane][a], y, acc);
            }
            scores[touched[i]] = (double)acc;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
constexpr int kSolveBlocks = 152 * 2;

// MTTKRP rows of the touched rows into Mc: FP64 rows of R indexed by row
// (TA = double), or compact FP32 rows of f32_row_stride(R) floats indexed by
// touched-row position (TA = float).
template <typename TA>
static int segmented_mttkrp(Session& s, cudaStream_t st) {
    const int R = s.R;
    const int hb = 152 * 8;
    if (std::is_same<TA, double>::value) {
        double* Mc = s.Mc;
        double* cf = s.carry_first;
        double* cl = s.carry_last;
        segreduce_kernel<double, double><<<hb, 256, 0, st>>>(R, s.counters, s.nnz, s.key_sorted, s.pay_sorted, s.ex_j,
                                                             s.ex_val, (const double*)s.D, Mc, cf, cl, s.carry_row);
        count_launch();
        segfix_kernel<double, kSegChunk><<<hb, 256, 0, st>>>(R, R, s.counters, s.nnz, s.carry_row, nullptr, nullptr,
                                                             s.key_sorted, cf, cl, Mc);
        count_launch();
    } else {
        const int RS = f32_row_stride(R), Q = RS / 4;
        float* Mc = reinterpret_cast<float*>(s.Mc);
        float* cf = reinterpret_cast<float*>(s.carry_first);
        float* cl = reinterpret_cast<float*>(s.carry_last);
        const float4* D4 = reinterpret_cast<const float4*>(s.Df);
#define EXAFAC_SEG_F32(QQ)                                                                                         \
    segreduce_f32_kernel<QQ><<<hb, 256, 0, st>>>(s.counters, s.nnz, s.key_sorted, s.pay64_sorted, s.chunk_seg, D4,     \
                                                 reinterpret_cast<float4*>(Mc), reinterpret_cast<float4*>(cf),      \
                                                 reinterpret_cast<float4*>(cl), s.carry_row, s.carry_seg)
        switch (Q) {
            case 1: EXAFAC_SEG_F32(1); break;
            case 2: EXAFAC_SEG_F32(2); break;
            case 3: EXAFAC_SEG_F32(3); break;
            case 4: EXAFAC_SEG_F32(4); break;
            case 5: EXAFAC_SEG_F32(5); break;
            case 6: EXAFAC_SEG_F32(6); break;
            case 7: EXAFAC_SEG_F32(7); break;
            default: EXAFAC_SEG_F32(8); break;
        }
#undef EXAFAC_SEG_F32
        count_launch();
        segfix_kernel<float, kSegChunkF32><<<hb, 256, 0, st>>>(R, RS, s.counters, s.nnz, s.carry_row, s.carry_seg,
                                                               s.seg_start, s.key_sorted, cf, cl, Mc);
        count_launch();
    }
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// ---------------------------------------------------------------------------
// FP32 forms of solve + Gram and normalize + leverage (mixed precisions).
// A warp owns 32 touched rows at a time, staged in shared memory with rows
// padded to KC floats (KC a multiple of 4, >= R):
//   * rows move between HBM and the tile one row per instruction (lane =
//     column), so each global access is one contiguous row; the solve reads
//     and writes compact rows (Mc, Uc), the normalisation writes the factor;
//   * row products run thread per row, the R x R operand read as float4
//     broadcasts from shared memory;
//   * the Gram of the solved rows is accumulated in 4 x 4 register blocks of
//     the lower triangle (NB blocks per lane), in FP32 within a 32-row tile
//     and in compensated FP32 (hi + lo) across tiles, then in FP64 over the
//     block's warps in warp
//     order (reproducible).
// ---------------------------------------------------------------------------
constexpr int kTileStride = 36;  // floats per staged row (16-byte aligned rows)

template <int KC>
struct TileShape {
    static constexpr int kBlk = KC / 4;                        // 4-column blocks per side
    static constexpr int kTri = kBlk * (kBlk + 1) / 2;         // lower-triangle blocks
    static constexpr int kNB = (kTri + 31) / 32;               // blocks per lane
};

template <int KC>
__global__ void __launch_bounds__(kSolveWarps * 32) solve_gram_f32_kernel(int R, const int64_t* __restrict__ counters,
                                                                         const float* __restrict__ Mc,
                                                                         const double* __restrict__ Phi,
                                                                         float* __restrict__ Uc,
                                                                         double* __restrict__ part) {
    using S = TileShape<KC>;
    __shared__ __align__(16) float phi[KC][KC];
    __shared__ __align__(16) float tile[kSolveWarps][32][kTileStride];  // at the end: the per-warp Gram slab
    static_assert(sizeof(tile) >= sizeof(float2) * kSolveWarps * (32 * 33 / 2), "slab does not fit");
    const int P = R * (R + 1) / 2;
    const int ldm = f32_row_stride(R);  // Mc row stride
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < KC * KC; e += blockDim.x) {
        const int a = e / KC, b = e % KC;
        phi[a][b] = (a < R && b < R) ? narrow_f64(Phi[a * R + b]) : 0.0f;
    }
    // this lane's lower-triangle 4x4 blocks
    int bi[S::kNB], bj[S::kNB];
#pragma unroll
    for (int q = 0; q < S::kNB; q++) {
        int blk = lane + 32 * q, i = 0;
        while (blk > i) {
            blk -= i + 1;
            i++;
        }
        bi[q] = (lane + 32 * q < S::kTri) ? i : -1;
        bj[q] = blk;
    }
    float ghi[S::kNB][16], glo[S::kNB][16];  // compensated sums over the warp's tiles
#pragma unroll
    for (int q = 0; q < S::kNB; q++)
#pragma unroll
        for (int x = 0; x < 16; x++) ghi[q][x] = glo[q][x] = 0.0f;
    __syncthreads();
    float (*t)[kTileStride] = tile[w];
    const int64_t nt = counters[2];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < nt; base += nwarps * 32) {
        const int nrow = (int)min((int64_t)32, nt - base);
        float v[32];  // stage M rows (compact: the tile is one contiguous block), zero padding
#pragma unroll
        for (int r = 0; r < 32; r++) v[r] = (r < nrow && lane < R) ? Mc[(base + r) * ldm + lane] : 0.0f;
#pragma unroll
        for (int r = 0; r < 32; r++)
            if (lane < KC) t[r][lane] = v[r];
        __syncwarp();
        float m[KC], u[KC];
#pragma unroll
        for (int c = 0; c < KC; c += 4) {
            const float4 v = *reinterpret_cast<const float4*>(&t[lane][c]);
            m[c] = v.x;
            m[c + 1] = v.y;
            m[c + 2] = v.z;
            m[c + 3] = v.w;
            u[c] = u[c + 1] = u[c + 2] = u[c + 3] = 0.0f;
        }
#pragma unroll
        for (int k = 0; k < KC; k++) {
            if (k < R) {
#pragma unroll
                for (int c = 0; c < KC; c += 4) {
                    const float4 p = *reinterpret_cast<const float4*>(&phi[k][c]);
                    u[c] = fmaf(m[k], p.x, u[c]);
                    u[c + 1] = fmaf(m[k], p.y, u[c + 1]);
                    u[c + 2] = fmaf(m[k], p.z, u[c + 2]);
                    u[c + 3] = fmaf(m[k], p.w, u[c + 3]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < KC; c += 4)
            *reinterpret_cast<float4*>(&t[lane][c]) = make_float4(u[c], u[c + 1], u[c + 2], u[c + 3]);
        __syncwarp();
        for (int r = 0; r < nrow; r++)  // store the solved rows, compact
            if (lane < ldm) Uc[(base + r) * ldm + lane] = t[r][lane];
#pragma unroll
        for (int q = 0; q < S::kNB; q++) {
            if (bi[q] >= 0) {
                float g[16];
#pragma unroll
                for (int x = 0; x < 16; x++) g[x] = 0.0f;
                for (int r = 0; r < 32; r++) {
                    const float4 a = *reinterpret_cast<const float4*>(&t[r][4 * bi[q]]);
                    const float4 b = *reinterpret_cast<const float4*>(&t[r][4 * bj[q]]);
                    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int x = 0; x < 4; x++)
#pragma unroll
                        for (int y = 0; y < 4; y++) g[x * 4 + y] = fmaf(av[x], bv[y], g[x * 4 + y]);
                }
#pragma unroll
                for (int x = 0; x < 16; x++) two_sum_acc(ghi[q][x], glo[q][x], g[x]);
            }
        }
        __syncwarp();
    }
    // Block sum in warp order: every warp leaves its (hi, lo) sums in its row
    // of a slab over the (now free) tiles, each packed entry with one owner
    // lane per warp; a thread per entry then adds the rows in order, still
    // compensated, and widens once.
    __syncthreads();
    float2* slab = reinterpret_cast<float2*>(&tile[0][0][0]);
#pragma unroll
    for (int q = 0; q < S::kNB; q++) {
        if (bi[q] < 0) continue;
#pragma unroll
        for (int x = 0; x < 4; x++)
#pragma unroll
            for (int y = 0; y < 4; y++) {
                const int a = 4 * bi[q] + x, b = 4 * bj[q] + y;  // b's block <= a's block
                if (a < R && b < R && b <= a)
                    slab[w * P + packed_index(R, b, a)] = make_float2(ghi[q][x * 4 + y], glo[q][x * 4 + y]);
            }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        float hi = 0.0f, lo = 0.0f;
#pragma unroll
        for (int ww = 0; ww < kSolveWarps; ww++) {
            const float2 v = slab[ww * P + e];
            two_sum_acc(hi, lo, v.x);
            lo += v.y;
        }
        part[(int64_t)blockIdx.x * P + e] = widen_f32(hi) + widen_f32(lo);
    }
}

// u_r = Uc_r / sigma (Uc: the compact rows of solve_gram_f32_kernel) written
// to U at the touched row, and, when P != null, l_r = u_r^T P u_r in FP32;
// rows staged as in solve_gram_f32_kernel.  This is the one scattered pass
// over the factor.  The scaling runs in FP32 (u = Uc * fl32(1 / sigma)) and
// the result is widened to FP64 exactly, so no element goes through the FP64
// pipe.
template <int KC>
__global__ void __launch_bounds__(kSolveWarps * 32) normlev_f32_kernel(int R, const int64_t* __restrict__ counters,
                                                                      const uint32_t* __restrict__ touched,
                                                                      const float* __restrict__ Uc,
                                                                      const double* __restrict__ sigma,
                                                                      const double* __restrict__ Pm,
                                                                      const int* __restrict__ degenerate,
                                                                      double* __restrict__ U,
                                                                      double* __restrict__ scores) {
    __shared__ __align__(16) float psm[KC][KC];
    __shared__ __align__(16) float tile[kSolveWarps][32][kTileStride];
    __shared__ float sg[32];
    // A zero column norm: write the unscaled rows and leave the division of
    // every row (as the reference does) to scale_rows_if_degenerate.
    const bool deg = *degenerate != 0;
    for (int e = threadIdx.x; e < KC * KC; e += blockDim.x) {
        const int a = e / KC, b = e % KC;
        psm[a][b] = (Pm && a < R && b < R) ? narrow_f64(Pm[a * R + b]) : 0.0f;
    }
    // Multiplying by fl32(1/sigma) differs from the reference's division by
    // at most two FP32 roundings.
    for (int c = threadIdx.x; c < 32; c += blockDim.x) sg[c] = deg ? 1.0f : (c < R ? (float)(1.0 / sigma[c]) : 0.0f);
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ldm = f32_row_stride(R);  // Uc row stride
    float (*t)[kTileStride] = tile[w];
    const float sgl = sg[lane];
    const int64_t nt = counters[2];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < nt; base += nwarps * 32) {
        const int nrow = (int)min((int64_t)32, nt - base);
        const uint32_t myrow = lane < nrow ? touched[base + lane] : 0u;
        {
            float v[32];  // the tile's compact rows (one contiguous block), all loads in flight
#pragma unroll
            for (int r = 0; r < 32; r++) v[r] = (r < nrow && lane < R) ? Uc[(base + r) * ldm + lane] : 0.0f;
#pragma unroll
            for (int r = 0; r < 32; r++)
                if (lane < KC) t[r][lane] = v[r];
        }
        __syncwarp();
        const uint32_t row0 = __shfl_sync(0xffffffffu, myrow, 0);
        const uint32_t row31 = __shfl_sync(0xffffffffu, myrow, 31);
        if (nrow == 32 && row31 - row0 == 31) {
            // 32 consecutive rows: one contiguous block of 32 R doubles, written
            // with full-width stores (lane l: elements l, l + 32, ...)
            double* blk = U + (int64_t)row0 * R;
            int r = lane / R, c = lane % R;
            for (int e = lane; e < 32 * R; e += 32) {
                const float y = t[r][c] * sg[c];
                blk[e] = widen_f32(y);
                t[r][c] = y;
                c += 32;
                while (c >= R) {
                    c -= R;
                    r++;
                }
            }
        } else {
#pragma unroll 4
            for (int r = 0; r < nrow; r++) {  // normalised FP64 rows to the factor, one row per store
                const int64_t row = __shfl_sync(0xffffffffu, myrow, r);
                if (lane < KC) {
                    const float y = t[r][lane] * sgl;
                    if (lane < R) U[row * R + lane] = widen_f32(y);
                    t[r][lane] = y;
                }
            }
        }
        __syncwarp();
        if (Pm && !deg && lane < nrow) {
            float u[KC];
#pragma unroll
            for (int c = 0; c < KC; c += 4) {
                const float4 v = *reinterpret_cast<const float4*>(&t[lane][c]);
                u[c] = v.x;
                u[c + 1] = v.y;
                u[c + 2] = v.z;
                u[c + 3] = v.w;
            }
            float acc = 0.0f;
#pragma unroll
            for (int a = 0; a < KC; a++) {
                if (a < R) {
                    float y = 0.0f;
#pragma unroll
                    for (int c = 0; c < KC; c += 4) {
                        const float4 p = *reinterpret_cast<const float4*>(&psm[a][c]);
                        y = fmaf(p.x, u[c], y);
                        y = fmaf(p.y, u[c + 1], y);
                        y = fmaf(p.z, u[c + 2], y);
                        y = fmaf(p.w, u[c + 3], y);
                    }
                    acc = fmaf(u[a], y, acc);
                }
            }
            scores[myrow] = widen_f32(acc);
        }
        __syncwarp();
    }
}

template <int KC>
static void launch_solve_f32(Session& s, int n, cudaStream_t st) {
    solve_gram_f32_kernel<KC><<<kSolveBlocks, kSolveWarps * 32, 0, st>>>(
        s.R, s.counters, reinterpret_cast<const float*>(s.Mc), s.dpinv, s.Uc, s.part);
}

template <int KC>
static void launch_normlev_f32(Session& s, int n, bool arls, cudaStream_t st) {
    normlev_f32_kernel<KC><<<kSolveBlocks, kSolveWarps * 32, 0, st>>>(
        s.R, s.counters, s.touched, s.Uc, s.F.sigma, arls ? s.upinv : nullptr, reinterpret_cast<int*>(s.counters + 6),
        s.F.U[n], arls ? s.scores[n] : nullptr);
}

static int solve_f32(Session& s, int n, cudaStream_t st) {
    EXAFAC_TRY(segmented_mttkrp<float>(s, st));
    EXAFAC_TRY(zero_factor_rows(s, n, st));
    if (s.R <= 16) launch_solve_f32<16>(s, n, st);
    else if (s.R <= 28) launch_solve_f32<28>(s, n, st);
    else launch_solve_f32<32>(s, n, st);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

template <typename TA>
static int solve_typed(Session& s, int n, cudaStream_t st) {
    const int R = s.R;
    EXAFAC_TRY(segmented_mttkrp<TA>(s, st));
    EXAFAC_TRY(zero_factor_rows(s, n, st));
    const int P = packed_size(R);
    const int Q = (P + 31) / 32;
    const TA* Mc = reinterpret_cast<const TA*>(s.Mc);
    if (Q <= 9) {
        const size_t smem = solve_gram_smem<TA, 9>();
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(solve_gram_kernel<TA, 9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        solve_gram_kernel<TA, 9><<<kSolveBlocks, kSolveWarps * 32, smem, st>>>(R, s.counters, s.touched, Mc, s.dpinv,
                                                                                s.F.U[n], s.part);
    } else {
        const size_t smem = solve_gram_smem<TA, 17>();
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(solve_gram_kernel<TA, 17>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        solve_gram_kernel<TA, 17><<<kSolveBlocks, kSolveWarps * 32, smem, st>>>(R, s.counters, s.touched, Mc,
                                                                                 s.dpinv, s.F.U[n], s.part);
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

template <typename TA>
static int normalize_typed(Session& s, int n, bool arls, cudaStream_t st) {
    const int R = s.R;
    EXAFAC_TRY(gram_reduce_to(s, kSolveBlocks, s.ugram, st));
    EXAFAC_TRY(sigma_and_gram(s, st));
    if (arls) EXAFAC_TRY(launch_pinv(R, s.ngram, s.upinv, 1e-11, s.vt, st));
    normlev_kernel<TA><<<grid_capped(s.dims[n], kNormWarps * 32), kNormWarps * 32, 0, st>>>(
        R, s.counters, s.touched, s.F.sigma, arls ? s.upinv : nullptr, reinterpret_cast<int*>(s.counters + 6),
        s.F.U[n], arls ? s.scores[n] : nullptr);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return scale_rows_if_degenerate(s, n, st);
}

int mttkrp_solve_balanced(Session& s, int n, cudaStream_t st) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) return solve_typed<double>(s, n, st);
    return solve_f32(s, n, st);
}

int normalize_balanced(Session& s, int n, bool arls, cudaStream_t st) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) return normalize_typed<double>(s, n, arls, st);
    const int R = s.R;
    EXAFAC_TRY(gram_reduce_to(s, kSolveBlocks, s.ugram, st));
    EXAFAC_TRY(sigma_and_gram(s, st));
    if (arls) EXAFAC_TRY(launch_pinv_leverage_f32(R, s.ngram, s.upinv, 1e-11, s.vt, st));
    if (R <= 16) launch_normlev_f32<16>(s, n, arls, st);
    else if (R <= 28) launch_normlev_f32<28>(s, n, arls, st);
    else launch_normlev_f32<32>(s, n, arls, st);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return scale_rows_if_degenerate(s, n, st);
}

__global__ void scatter_rows_kernel(int R, const int64_t* __restrict__ counters, const uint32_t* __restrict__ touched,
                                    const double* __restrict__ Mc, double* __restrict__ out) {
    const int64_t nt = counters[2];
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nt * R; e += (int64_t)gridDim.x * blockDim.x)
        out[(int64_t)touched[e / R] * R + e % R] = Mc[(int64_t)touched[e / R] * R + e % R];
}

// MTTKRP rows (FP64) written to a dense dims[n] x R output (zeroed by the caller).
int mttkrp_scatter_out(Session& s, double* out, cudaStream_t st) {
    EXAFAC_TRY(segmented_mttkrp<double>(s, st));
    scatter_rows_kernel<<<152 * 8, 256, 0, st>>>(s.R, s.counters, s.touched, s.Mc, out);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

}  // namespace exafac
