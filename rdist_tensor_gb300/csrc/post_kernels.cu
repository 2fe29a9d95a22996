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
#include "bulk.cuh"
#include "dense.cuh"
#include "engine.cuh"
#include "segfix.cuh"
#include "mma.cuh"
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
// hits per instruction.  Each lane loads its share of the group's hits (row and
// the packed (sample, value) that travelled through the sort) for every 8
// of the chunk; hit t of the chunk is broadcast from lane t % 8 of the group.  Design rows are gathered 8 hits at a time before their FMAs.  Rows
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
    pdl_trigger();
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
        // this lane's hit of the round (hit b + sub), loaded one round ahead
        auto load_hit = [&](int t, uint32_t& r, uint32_t& j, float& v) {
            r = kNoRow;
            j = 0;
            v = 0.f;
            if (t < n) {
                r = keys[cs + t];
                const uint64_t p = pay64[cs + t];
                j = (uint32_t)p;
                v = __uint_as_float((uint32_t)(p >> 32));
            }
        };
        uint32_t nr_, nj_;
        float nv_;
        load_hit(sub, nr_, nj_, nv_);
        uint32_t cur = __shfl_sync(gmask, nr_, 0, 8);
        int64_t seg = chunk_seg[c];  // compact index of the run holding hit cs
        bool first_seg = true;
        float4 acc = zero4;
#pragma unroll 1
        for (int b = 0; b < C && b < n; b += 8) {
            const uint32_t hr = nr_, hj = nj_;
            const float hv = nv_;
            if (b + 8 < C) load_hit(b + 8 + sub, nr_, nj_, nv_);
            float4 d[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const uint32_t jt = __shfl_sync(gmask, hj, u, 8);
                d[u] = (b + u < n && col) ? D4[(int64_t)jt * 8 + sub] : zero4;  // 128-byte rows
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int t = b + u;
                const uint32_t rt = __shfl_sync(gmask, hr, u, 8);
                const float vt = __shfl_sync(gmask, hv, u, 8);
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
                                                                 double* __restrict__ U, double* __restrict__ scores,
                                                                 double* __restrict__ scores_c) {
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
            scores_c[i] = (double)acc;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
constexpr int kSolveBlocks = 152 * 2;
constexpr int kNormlevBlocks = 152 * 4;  // no per-block partials: four resident blocks per SM (64 registers)

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
        EXAFAC_CUDA_TRY(launch_dependent(segfix_kernel<float, kSegChunkF32>, hb, 256, 0, st, R, RS, s.counters, s.nnz,
                                         s.carry_row, s.carry_seg, s.seg_start, s.key_sorted, cf, cl, Mc));
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

// The FP32 solve on the tensor cores: per 32-row tile of compact M rows,
// U = M Phi and the tile's Gram U^T U as mma.sync m16n8k8 products in 3xTF32
// (each operand split as hi + lo, products hi*hi + hi*lo + lo*hi with FP32
// accumulation: about 2^-21 relative, near FP32's own rounding), the Gram
// summed over a warp's tiles in compensated FP32 and over the block's warps
// in warp order (reproducible).  A warp owns a tile at a time:
//   * the M tile (32 compact rows, contiguous) arrives by one bulk copy into
//     Mbuf, rows of ldm floats as in Mc, the next tile's copy being issued as
//     soon as this tile's M has been read (columns past ldm of a fragment
//     are masked to zero);
//   * U goes to two tiles, Th = TF32(U) and Tl = U - Th (exact), which hold
//     the Gram's operands ready-split and give U back as Th + Tl for Uc.
// Mbuf rows are ldm floats (the A-fragment loads are conflict-free when
// ldm / 4 is odd, e.g. 28); Th and Tl rows are 8 KT + 4 floats.  Phi is held
// split (hi, lo) with rows of 8 KT + 8 floats, for conflict-free B-fragment
// loads.
constexpr int kMmaWarps = 4;
constexpr int kMmaBlocks = 152 * 3;

template <int KC>
struct MmaShape {
    static constexpr int KT = (KC + 7) / 8;       // k-steps of the product and its n-tiles (8 KT >= R)
    static constexpr int GM = (KC + 15) / 16;     // 16-row m-tiles of the Gram
    static constexpr int kPairs = GM == 1 ? 2 : 6;  // lower-triangle (m-tile, n-tile) blocks of the Gram
    static constexpr int kStride = 8 * KT + 4;
    static constexpr int kPhiStride = 8 * KT + 8;
    static constexpr size_t kTileBytes = sizeof(float) * 32 * kStride;
    static constexpr size_t kWarpBytes = 3 * kTileBytes;  // Mbuf, Th, Tl
    static constexpr size_t kSmem = kMmaWarps * kWarpBytes + 2 * sizeof(float) * (8 * KT) * kPhiStride;
};

template <int KC>
__global__ void __launch_bounds__(kMmaWarps * 32) solve_gram_mma_kernel(int R, const int64_t* __restrict__ counters,
                                                                        const float* __restrict__ Mc,
                                                                        const double* __restrict__ Phi,
                                                                        float* __restrict__ Uc,
                                                                        double* __restrict__ part,
                                                                        DeviceStatus* err) {
    using S = MmaShape<KC>;
    constexpr int KT = S::KT, TS = S::kStride, PS = S::kPhiStride, KP = 8 * KT;
    extern __shared__ __align__(128) unsigned char mma_dyn[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    float* Mbuf = reinterpret_cast<float*>(mma_dyn + w * S::kWarpBytes);  // rows of ldm floats
    float (*Th)[TS] = reinterpret_cast<float (*)[TS]>(mma_dyn + w * S::kWarpBytes + S::kTileBytes);
    float (*Tl)[TS] = reinterpret_cast<float (*)[TS]>(mma_dyn + w * S::kWarpBytes + 2 * S::kTileBytes);
    float (*phh)[PS] = reinterpret_cast<float (*)[PS]>(mma_dyn + kMmaWarps * S::kWarpBytes);
    float (*phl)[PS] = phh + KP;
    __shared__ __align__(8) uint64_t bars[kMmaWarps];
    __shared__ int copy_pending;  // a warp left with a bulk copy still landing in its tiles
    if (threadIdx.x == 0) copy_pending = 0;
    pdl_wait();
    pdl_trigger();
    const int P = R * (R + 1) / 2;
    const int ldm = f32_row_stride(R);  // Mc / Uc row stride
    const uint32_t row_bytes = (uint32_t)(sizeof(float) * ldm);
    for (int e = threadIdx.x; e < KP * KP; e += blockDim.x) {
        const int a = e / KP, b = e % KP;
        const float x = (a < R && b < R) ? narrow_f64(Phi[a * R + b]) : 0.0f;
        uint32_t hi, lo;
        split_tf32(x, hi, lo);
        phh[a][b] = __uint_as_float(hi);
        phl[a][b] = __uint_as_float(lo);
    }
    {  // zero the warp's tiles once
        float* z = Mbuf;
        for (int e = lane; e < 3 * 32 * TS; e += 32) z[e] = 0.0f;
    }
    if (lane == 0) mbar_init(&bars[w], 1);
    fence_proxy_async_smem();
    __syncthreads();
    const int64_t nt = counters[2];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    auto issue = [&](int64_t b) {  // one copy of the tile's nr contiguous rows
        const int nr = (int)min((int64_t)32, nt - b);
        if (lane == 0) {
            mbar_arrive_expect_tx(&bars[w], row_bytes * (uint32_t)nr);
            bulk_g2s(Mbuf, Mc + b * ldm, row_bytes * (uint32_t)nr, &bars[w]);
        }
    };
    float ghi[S::kPairs][4], glo[S::kPairs][4];  // compensated sums over the warp's tiles
#pragma unroll
    for (int p = 0; p < S::kPairs; p++)
#pragma unroll
        for (int i = 0; i < 4; i++) ghi[p][i] = glo[p][i] = 0.0f;
    uint32_t phase = 0;
    int64_t base = warp * 32;
    if (base < nt) issue(base);
    for (; base < nt; base += nwarps * 32) {
        const int nrow = (int)min((int64_t)32, nt - base);
        if (!mbar_wait(&bars[w], phase)) {  // (the block still meets its barriers)
            if (lane == 0) report(err, EXAFAC_ERR_TIMEOUT, 10, base, nt);
            // the tile's copy is the warp's only one in flight (the next is
            // issued after this tile is consumed): give it one more bounded
            // wait before the warp leaves its shared memory; if that runs out
            // too, the block leaves its tiles alone (no slab reduction)
            if (!mbar_wait(&bars[w], phase) && lane == 0) copy_pending = 1;
            break;
        }
        phase ^= 1u;
        for (int e = nrow * ldm + lane; e < 32 * ldm; e += 32) Mbuf[e] = 0.0f;  // rows past a short tile's end
        __syncwarp();
        // U = M Phi
        float acc[2][KT][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt8 = 0; nt8 < KT; nt8++)
#pragma unroll
                for (int i = 0; i < 4; i++) acc[mt][nt8][i] = 0.0f;
#pragma unroll
        for (int ks = 0; ks < KT; ks++) {
            uint32_t ah[2][4], al[2][4];
            const int c0 = 8 * ks + tig, c1 = c0 + 4;  // columns; past ldm they read the next row: masked
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                const float* r0 = Mbuf + (16 * mt + gid) * ldm;
                const float* r1 = r0 + 8 * ldm;
                split_tf32(c0 < ldm ? r0[c0] : 0.0f, ah[mt][0], al[mt][0]);
                split_tf32(c0 < ldm ? r1[c0] : 0.0f, ah[mt][1], al[mt][1]);
                split_tf32(c1 < ldm ? r0[c1] : 0.0f, ah[mt][2], al[mt][2]);
                split_tf32(c1 < ldm ? r1[c1] : 0.0f, ah[mt][3], al[mt][3]);
            }
#pragma unroll
            for (int nt8 = 0; nt8 < KT; nt8++) {
                const uint32_t bh[2] = {__float_as_uint(phh[8 * ks + tig][8 * nt8 + gid]),
                                        __float_as_uint(phh[8 * ks + tig + 4][8 * nt8 + gid])};
                const uint32_t bl[2] = {__float_as_uint(phl[8 * ks + tig][8 * nt8 + gid]),
                                        __float_as_uint(phl[8 * ks + tig + 4][8 * nt8 + gid])};
#pragma unroll
                for (int mt = 0; mt < 2; mt++) {
                    mma_tf32_16x8x8(acc[mt][nt8], al[mt], bh);
                    mma_tf32_16x8x8(acc[mt][nt8], ah[mt], bl);
                    mma_tf32_16x8x8(acc[mt][nt8], ah[mt], bh);
                }
            }
        }
        __syncwarp();  // the M tile is consumed: the next tile's copies may land
        if (base + nwarps * 32 < nt) {
            fence_proxy_async_smem();
            issue(base + nwarps * 32);
        }
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt8 = 0; nt8 < KT; nt8++)
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int row = 16 * mt + gid + 8 * (i >> 1), col = 8 * nt8 + 2 * tig + (i & 1);
                    uint32_t hi, lo;
                    split_tf32(acc[mt][nt8][i], hi, lo);
                    Th[row][col] = __uint_as_float(hi);
                    Tl[row][col] = __uint_as_float(lo);
                }
        __syncwarp();
        for (int r = 0; r < nrow; r++)  // the solved rows, compact (hi + lo = U exactly)
            if (lane < ldm) Uc[(base + r) * ldm + lane] = Th[r][lane] + Tl[r][lane];
        // the tile's Gram: A = U^T (rows = columns of U), B = U, K = the 32 rows
        float g[S::kPairs][4];
#pragma unroll
        for (int p = 0; p < S::kPairs; p++)
#pragma unroll
            for (int i = 0; i < 4; i++) g[p][i] = 0.0f;
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {
            const int k0 = 8 * ks + tig;
            uint32_t ah[S::GM][4], al[S::GM][4], bh[2 * S::GM][2], bl[2 * S::GM][2];
#pragma unroll
            for (int mt = 0; mt < S::GM; mt++) {
                ah[mt][0] = __float_as_uint(Th[k0][16 * mt + gid]);
                ah[mt][1] = __float_as_uint(Th[k0][16 * mt + gid + 8]);
                ah[mt][2] = __float_as_uint(Th[k0 + 4][16 * mt + gid]);
                ah[mt][3] = __float_as_uint(Th[k0 + 4][16 * mt + gid + 8]);
                al[mt][0] = __float_as_uint(Tl[k0][16 * mt + gid]);
                al[mt][1] = __float_as_uint(Tl[k0][16 * mt + gid + 8]);
                al[mt][2] = __float_as_uint(Tl[k0 + 4][16 * mt + gid]);
                al[mt][3] = __float_as_uint(Tl[k0 + 4][16 * mt + gid + 8]);
            }
#pragma unroll
            for (int nt8 = 0; nt8 < 2 * S::GM; nt8++) {
                bh[nt8][0] = __float_as_uint(Th[k0][8 * nt8 + gid]);
                bh[nt8][1] = __float_as_uint(Th[k0 + 4][8 * nt8 + gid]);
                bl[nt8][0] = __float_as_uint(Tl[k0][8 * nt8 + gid]);
                bl[nt8][1] = __float_as_uint(Tl[k0 + 4][8 * nt8 + gid]);
            }
#pragma unroll
            for (int p = 0; p < S::kPairs; p++) {
                const int mt = p < 2 ? 0 : 1, nt8 = p < 2 ? p : p - 2;
                mma_tf32_16x8x8(g[p], al[mt], bh[nt8]);
                mma_tf32_16x8x8(g[p], ah[mt], bl[nt8]);
                mma_tf32_16x8x8(g[p], ah[mt], bh[nt8]);
            }
        }
#pragma unroll
        for (int p = 0; p < S::kPairs; p++)
#pragma unroll
            for (int i = 0; i < 4; i++) two_sum_acc(ghi[p][i], glo[p][i], g[p][i]);
        __syncwarp();
    }
    // Block sum in warp order: every warp leaves its (hi, lo) sums in its row
    // of a slab over the (now idle) tiles, each packed entry with one owner
    // lane per warp; a thread per entry then adds the rows in order, still
    // compensated, and widens once.
    __syncthreads();
    if (copy_pending) return;  // uniform: read after the barrier; the step's error is reported
    float2* slab = reinterpret_cast<float2*>(mma_dyn);
    static_assert(kMmaWarps * S::kWarpBytes >= sizeof(float2) * kMmaWarps * (KC * (KC + 1) / 2), "slab");
#pragma unroll
    for (int p = 0; p < S::kPairs; p++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int mt = p < 2 ? 0 : 1, nt8 = p < 2 ? p : p - 2;
            const int row = 16 * mt + gid + 8 * (i >> 1), col = 8 * nt8 + 2 * tig + (i & 1);
            if (row < R && col <= row) slab[w * P + packed_index(R, col, row)] = make_float2(ghi[p][i], glo[p][i]);
        }
    __syncthreads();
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        float hi = 0.0f, lo = 0.0f;
#pragma unroll
        for (int ww = 0; ww < kMmaWarps; ww++) {
            const float2 v = slab[ww * P + e];
            two_sum_acc(hi, lo, v.x);
            lo += v.y;
        }
        part[(int64_t)blockIdx.x * P + e] = widen_f32(hi) + widen_f32(lo);
    }
}

// u_r = Uc_r / sigma (Uc: the compact rows of solve_gram_mma_kernel) written
// to U at the touched row, and, when P != null, l_r = u_r^T P u_r in FP32;
// rows staged in shared memory, 32 per warp.  This is the one scattered pass
// over the factor.  The scaling runs in FP32 (u = Uc * fl32(1 / sigma)); the
// result is widened to FP64 by the hardware conversion, one FP64-pipe
// operation per element: this kernel is bound by instruction issue, and the
// conversions' FP64-pipe time stays well below its run time (the integer
// widening would cost seven issue slots).
constexpr int kTileStride = 36;  // floats per staged row of normlev_f32_kernel (16-byte aligned rows)

template <int KC>
__global__ void __launch_bounds__(kSolveWarps * 32, 4) normlev_f32_kernel(int R, const int64_t* __restrict__ counters,
                                                                      const uint32_t* __restrict__ touched,
                                                                      const float* __restrict__ Uc,
                                                                      const double* __restrict__ sigma,
                                                                      const double* __restrict__ Pm,
                                                                      const int* __restrict__ degenerate,
                                                                      double* __restrict__ U,
                                                                      double* __restrict__ scores,
                                                                      double* __restrict__ scores_c) {
    __shared__ __align__(16) float psm[KC][KC];
    __shared__ __align__(16) float tile[kSolveWarps][32][kTileStride];
    __shared__ float sg[32];
    pdl_wait();
    pdl_trigger();
    // A zero column norm: write the unscaled rows and leave the division of
    // every row (as the reference does) to scale_rows_if_degenerate.
    const bool deg = *degenerate != 0;
    for (int e = threadIdx.x; e < KC * KC; e += blockDim.x) {
        const int a = e / KC, b = e % KC;
        // upper triangle, off-diagonal entries doubled (u^T P u with P symmetric)
        psm[a][b] = (Pm && a < R && b < R && b >= a) ? narrow_f64((b == a ? 1.0 : 2.0) * Pm[a * R + b]) : 0.0f;
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
                blk[e] = (double)y;
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
                    if (lane < R) U[row * R + lane] = (double)y;
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
            // u^T P u over the upper triangle: psm holds P_aa on the diagonal,
            // 2 P_ac above it and zeros below, so row a needs only the
            // 4-column groups from a's own onwards
            float acc = 0.0f;
#pragma unroll
            for (int a = 0; a < KC; a++) {
                if (a < R) {
                    float y = 0.0f;
#pragma unroll
                    for (int c = (a / 4) * 4; c < KC; c += 4) {
                        const float4 p = *reinterpret_cast<const float4*>(&psm[a][c]);
                        y = fmaf(p.x, u[c], y);
                        y = fmaf(p.y, u[c + 1], y);
                        y = fmaf(p.z, u[c + 2], y);
                        y = fmaf(p.w, u[c + 3], y);
                    }
                    acc = fmaf(u[a], y, acc);
                }
            }
            const double l = (double)acc;
            scores[myrow] = l;
            scores_c[base + lane] = l;  // by touched-row index, for the CDF
        }
        __syncwarp();
    }
}

template <int KC>
static int launch_solve_f32(Session& s, int n, cudaStream_t st) {
    const size_t smem = MmaShape<KC>::kSmem;
    EXAFAC_CUDA_TRY(
        cudaFuncSetAttribute(solve_gram_mma_kernel<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // follows segfix, unless a dense factor was cleared in between
    EXAFAC_CUDA_TRY(launch_dependent_if(!s.dense[n], solve_gram_mma_kernel<KC>, kMmaBlocks, kMmaWarps * 32, smem, st,
                                        s.R, s.counters, reinterpret_cast<const float*>(s.Mc), s.dpinv, s.Uc, s.part,
                                        s.status));
    return EXAFAC_OK;
}

template <int KC>
static int launch_normlev_f32(Session& s, int n, bool arls, cudaStream_t st) {
    EXAFAC_CUDA_TRY(launch_dependent(normlev_f32_kernel<KC>, kNormlevBlocks, kSolveWarps * 32, 0, st, s.R, s.counters,
                                     s.touched, (const float*)s.Uc, s.F.sigma, arls ? s.upinv : nullptr,
                                     reinterpret_cast<int*>(s.counters + 6), s.F.U[n], arls ? s.scores[n] : nullptr,
                                     s.scores_c));
    return EXAFAC_OK;
}

static int solve_f32(Session& s, int n, cudaStream_t st) {
    EXAFAC_TRY(segmented_mttkrp<float>(s, st));
    EXAFAC_TRY(clear_dense_factor(s, n, st));  // the old rows are cleared beside the update
    if (s.R <= 16) EXAFAC_TRY(launch_solve_f32<16>(s, n, st));
    else if (s.R <= 28) EXAFAC_TRY(launch_solve_f32<28>(s, n, st));
    else EXAFAC_TRY(launch_solve_f32<32>(s, n, st));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

template <typename TA>
static int solve_typed(Session& s, int n, cudaStream_t st) {
    const int R = s.R;
    EXAFAC_TRY(segmented_mttkrp<TA>(s, st));
    EXAFAC_TRY(clear_dense_factor(s, n, st));  // the old rows are cleared beside the update
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
        s.F.U[n], arls ? s.scores[n] : nullptr, s.scores_c);
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
    EXAFAC_TRY(gram_reduce_to(s, kMmaBlocks, s.ugram, st));
    if (arls)
        EXAFAC_TRY(launch_sigma_pinv_f32(R, s.ugram, s.F.sigma, s.ngram, reinterpret_cast<int*>(s.counters + 6),
                                         s.upinv, 1e-11, s.vt, st));
    else
        EXAFAC_TRY(sigma_and_gram(s, st));
    if (R <= 16) EXAFAC_TRY(launch_normlev_f32<16>(s, n, arls, st));
    else if (R <= 28) EXAFAC_TRY(launch_normlev_f32<28>(s, n, arls, st));
    else EXAFAC_TRY(launch_normlev_f32<32>(s, n, arls, st));
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
