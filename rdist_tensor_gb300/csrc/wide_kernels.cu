// Sampled MTTKRP, solve and renormalisation for 32 < R <= 128
// (csr_based_spmm scatter half sort_lookup.hpp:347-371, parallel_dsymm
// accumulator_stationary.hpp:283-286, DistMat1D::renormalize_columns
// distmat.hpp:85-138), in one arithmetic type T for the whole chain:
// T = double for the FP64 form, T = float for the mixed forms (their design
// rows are FP32, their hits carry FP32 values through the row sort).
//
//   1. segreduce_wide_kernel: warp per 64-hit chunk of the row-sorted hits,
//      lane l holding columns l + 32 c (c < CB); design rows of 8 hits are
//      gathered before their FMAs; rows inside a chunk go to M (compact, by
//      touched-row index), rows that cross a chunk border leave carries that
//      segfix_kernel adds in chunk order (the sums have a fixed order).
//   2. solve_gram_wide_kernel: U = M Phi over 32-row tiles, Phi and the tile
//      staged in shared memory, 4 rows x CB columns per thread; the tile's
//      Gram U^T U in 4 x 4 register blocks of its lower triangle, summed over
//      the block's tiles (compensated in FP32, plain in FP64) and written per
//      block in a fixed order.
//   3. normalize_wide_kernel: u = U / sigma written to the factor's touched
//      rows in FP64 and, for CP-ARLS-LEV, the leverage u^T P u.
#include "dense.cuh"
#include "engine.cuh"
#include "prims.cuh"
#include "segfix.cuh"

namespace exafac {

constexpr int kWideChunk = kSegChunkF32;  // 64 hits; chunk_seg is recorded per 64 hits by the run pass
constexpr int kWideWarps = 8;
constexpr int kWideSolveBlocks = 152;
constexpr int kWideTileRows = 32;

__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += e;
}

template <typename T>
struct WideHit {
    uint32_t row, sample;
    T value;
};

// Hit t of the row-sorted list: (row, sample, value).  FP64 form: the
// payload is the hit's index into ex_j / ex_val; mixed forms: the payload
// packs (sample, FP32 value).
template <typename T>
__device__ __forceinline__ WideHit<T> load_hit(int64_t t, const uint32_t* __restrict__ keys,
                                               const uint32_t* __restrict__ pay, const uint32_t* __restrict__ ex_j,
                                               const double* __restrict__ ex_val, const uint64_t* __restrict__ pay64) {
    WideHit<T> h;
    h.row = keys[t];
    if (pay64) {
        const uint64_t p = pay64[t];
        h.sample = (uint32_t)p;
        h.value = (T)__uint_as_float((uint32_t)(p >> 32));
    } else {
        const uint32_t i = pay[t];
        h.sample = ex_j[i];
        h.value = (T)ex_val[i];
    }
    return h;
}

template <typename T, int CB>
__global__ void __launch_bounds__(256) segreduce_wide_kernel(int R, int ldd, int ldm, const int64_t* __restrict__ counters,
                                                             int64_t cap, const uint32_t* __restrict__ keys,
                                                             const uint32_t* __restrict__ pay,
                                                             const uint32_t* __restrict__ ex_j,
                                                             const double* __restrict__ ex_val,
                                                             const uint64_t* __restrict__ pay64,
                                                             const uint32_t* __restrict__ chunk_seg,
                                                             const T* __restrict__ D, T* __restrict__ Mc,
                                                             T* __restrict__ carry_first, T* __restrict__ carry_last,
                                                             uint32_t* __restrict__ carry_row,
                                                             uint32_t* __restrict__ carry_seg) {
    pdl_wait();
    pdl_trigger();
    constexpr int C = kWideChunk;
    constexpr int CS = 32 * CB;  // carry stride
    const int64_t H = min(counters[1], cap);
    const int64_t nchunks = (H + C - 1) / C;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned full = 0xffffffffu;
    for (int64_t c = warp; c < nchunks; c += nwarps) {
        const int64_t cs = c * C;
        const int n = (int)min((int64_t)C, H - cs);
        const uint32_t prev_row = cs > 0 ? keys[cs - 1] : kNoRow;
        const uint32_t next_row = cs + n < H ? keys[cs + n] : kNoRow;
        uint32_t cur = keys[cs];
        int64_t seg = chunk_seg[c];  // touched-row index of the run holding hit cs
        bool first_seg = true;
        T acc[CB];
#pragma unroll
        for (int b = 0; b < CB; b++) acc[b] = T(0);
        auto flush = [&](bool to_first) {
#pragma unroll
            for (int b = 0; b < CB; b++) {
                const int col = lane + 32 * b;
                if (col < R) {
                    if (to_first) carry_first[c * CS + col] = acc[b];
                    else Mc[seg * ldm + col] = acc[b];
                }
            }
        };
#pragma unroll 1
        for (int g = 0; g < n; g += 32) {
            const int m = min(32, n - g);
            WideHit<T> h{kNoRow, 0u, T(0)};
            if (lane < m) h = load_hit<T>(cs + g + lane, keys, pay, ex_j, ex_val, pay64);
#pragma unroll 1
            for (int u0 = 0; u0 < m; u0 += 8) {
                T d[8][CB];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const uint32_t jt = __shfl_sync(full, h.sample, u0 + u);
#pragma unroll
                    for (int b = 0; b < CB; b++) {
                        const int col = lane + 32 * b;
                        d[u][b] = (u0 + u < m && col < R) ? D[(int64_t)jt * ldd + col] : T(0);
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const uint32_t rt = __shfl_sync(full, h.row, u0 + u);
                    const T vt = __shfl_sync(full, h.value, u0 + u);
                    if (u0 + u < m) {
                        if (rt != cur) {  // the open segment ends inside the chunk
                            flush(first_seg && cur == prev_row);
                            first_seg = false;
                            cur = rt;
                            seg++;
#pragma unroll
                            for (int b = 0; b < CB; b++) acc[b] = T(0);
                        }
#pragma unroll
                        for (int b = 0; b < CB; b++) acc[b] = fmat(d[u][b], vt, acc[b]);
                    }
                }
            }
        }
        const bool started_before = first_seg && cur == prev_row;
        const bool continues = cur == next_row;
        if (started_before) {
            flush(true);
        } else if (continues) {
#pragma unroll
            for (int b = 0; b < CB; b++) {
                const int col = lane + 32 * b;
                if (col < R) carry_last[c * CS + col] = acc[b];
            }
        } else {
            flush(false);
        }
        if (lane == 0) {
            carry_row[c] = (!started_before && continues) ? cur : kNoRow;
            carry_seg[c] = (uint32_t)seg;
        }
    }
}

// Lower-triangle 4 x 4 blocks of an R x R Gram handled by one thread.
constexpr int kGramBlocksPerThread = 3;  // ceil(528 / 256) at R = 128

template <typename T>
struct GramAcc;
template <>
struct GramAcc<float> {
    float hi[kGramBlocksPerThread][16], lo[kGramBlocksPerThread][16];
    __device__ void zero() {
#pragma unroll
        for (int q = 0; q < kGramBlocksPerThread; q++)
#pragma unroll
            for (int i = 0; i < 16; i++) hi[q][i] = lo[q][i] = 0.0f;
    }
    __device__ void add(int q, int i, float x) { two_sum_add(hi[q][i], lo[q][i], x); }
    __device__ double get(int q, int i) const { return widen_f32(hi[q][i]) + widen_f32(lo[q][i]); }
};
template <>
struct GramAcc<double> {
    double v[kGramBlocksPerThread][16];
    __device__ void zero() {
#pragma unroll
        for (int q = 0; q < kGramBlocksPerThread; q++)
#pragma unroll
            for (int i = 0; i < 16; i++) v[q][i] = 0.0;
    }
    __device__ void add(int q, int i, double x) { v[q][i] += x; }
    __device__ double get(int q, int i) const { return v[q][i]; }
};

// Block index q -> (block row, block col) of the lower triangle, row-major.
__device__ __forceinline__ void tri_block(int q, int& br, int& bc) {
    int r = (int)((sqrtf(8.0f * q + 1.0f) - 1.0f) * 0.5f);
    while ((r + 1) * (r + 2) / 2 <= q) r++;
    while (r * (r + 1) / 2 > q) r--;
    br = r;
    bc = q - r * (r + 1) / 2;
}

// U = M Phi for the touched rows (M compact, row stride ldm) and the Gram of
// U.  FP64 form (Uc == null): U goes to the factor's touched rows, FP64.
// Mixed forms: U goes to Uc (compact, stride ldm).  Dynamic shared memory:
// Phi [R][RP] then the tile [32][RP + 4] (RP = 32 CB, zero padded).
template <typename T, int CB>
__global__ void __launch_bounds__(kWideWarps * 32) solve_gram_wide_kernel(int R, int ldm,
                                                                          const int64_t* __restrict__ counters,
                                                                          const uint32_t* __restrict__ touched,
                                                                          const T* __restrict__ Mc,
                                                                          const double* __restrict__ Phi,
                                                                          double* __restrict__ U, T* __restrict__ Uc,
                                                                          double* __restrict__ part) {
    constexpr int RP = 32 * CB;
    constexpr int TS = RP + 4;  // tile row stride (16-byte aligned rows, fewer bank conflicts)
    extern __shared__ __align__(16) unsigned char wide_dyn[];
    T* phi = reinterpret_cast<T*>(wide_dyn);
    T* tile = phi + RP * RP;
    pdl_wait();
    pdl_trigger();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < RP * RP; e += blockDim.x) {
        const int a = e / RP, b = e % RP;
        phi[e] = (a < R && b < R) ? (T)Phi[a * R + b] : T(0);
    }
    const int nbr = (R + 3) / 4;
    const int nblk = nbr * (nbr + 1) / 2;
    GramAcc<T> gacc;
    gacc.zero();
    const int64_t nt = counters[2];
    const int64_t ntiles = (nt + kWideTileRows - 1) / kWideTileRows;
    for (int64_t tile_i = blockIdx.x; tile_i < ntiles; tile_i += gridDim.x) {
        const int64_t base = tile_i * kWideTileRows;
        const int rows = (int)min((int64_t)kWideTileRows, nt - base);
        __syncthreads();  // Phi is staged / the previous tile's Gram is done
        for (int e = threadIdx.x; e < kWideTileRows * RP; e += blockDim.x) {
            const int r = e / RP, col = e % RP;
            tile[r * TS + col] = (r < rows && col < R) ? Mc[(base + r) * ldm + col] : T(0);
        }
        __syncthreads();
        // rows 4w .. 4w+3, columns lane + 32 b
        T acc[4][CB];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int b = 0; b < CB; b++) acc[i][b] = T(0);
        const T* mrow = tile + (4 * w) * TS;
#pragma unroll 4
        for (int k = 0; k < R; k++) {
            T p[CB];
#pragma unroll
            for (int b = 0; b < CB; b++) p[b] = phi[k * RP + lane + 32 * b];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const T m = mrow[i * TS + k];
#pragma unroll
                for (int b = 0; b < CB; b++) acc[i][b] = fmat(m, p[b], acc[i][b]);
            }
        }
        __syncthreads();  // every warp has read its M rows: the tile now takes U
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int r = 4 * w + i;
#pragma unroll
            for (int b = 0; b < CB; b++) {
                const int col = lane + 32 * b;
                tile[r * TS + col] = (r < rows) ? acc[i][b] : T(0);
                if (r < rows && col < R) {
                    if (Uc) Uc[(base + r) * ldm + col] = acc[i][b];
                    else U[(int64_t)touched[base + r] * R + col] = (double)acc[i][b];
                }
            }
        }
        __syncthreads();
        // the tile's Gram, 4 x 4 blocks of the lower triangle
#pragma unroll
        for (int q = 0; q < kGramBlocksPerThread; q++) {
            const int bq = threadIdx.x + q * (kWideWarps * 32);
            if (bq >= nblk) continue;
            int br, bc;
            tri_block(bq, br, bc);
            T g[16];
#pragma unroll
            for (int i = 0; i < 16; i++) g[i] = T(0);
            for (int r = 0; r < kWideTileRows; r++) {
                const T* u = tile + r * TS;
                T ua[4], ub[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    ua[i] = u[4 * br + i];
                    ub[i] = u[4 * bc + i];
                }
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) g[i * 4 + j] = fmat(ua[i], ub[j], g[i * 4 + j]);
            }
#pragma unroll
            for (int i = 0; i < 16; i++) gacc.add(q, i, g[i]);
        }
    }
    // the block's Gram, packed upper triangle (entry (a, b), a <= b, from the
    // lower-triangle block holding (b, a))
    const int P = packed_size(R);
#pragma unroll
    for (int q = 0; q < kGramBlocksPerThread; q++) {
        const int bq = threadIdx.x + q * (kWideWarps * 32);
        if (bq >= nblk) continue;
        int br, bc;
        tri_block(bq, br, bc);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int row = 4 * br + i, col = 4 * bc + j;  // row >= col in the lower triangle
                if (row < R && col <= row) part[(int64_t)blockIdx.x * P + packed_index(R, col, row)] = gacc.get(q, i * 4 + j);
            }
    }
}

// u = U / sigma for the touched rows, written to the factor in FP64, and for
// CP-ARLS-LEV l = u^T P u (P the pseudo-inverse of the normalised Gram) into
// scores (by row) and scores_c (by touched-row index).  Warp per row, lane l
// holding columns l + 32 c.  FP64 form: U is read from the factor in place;
// mixed forms: from Uc (compact FP32).  The leverage is formed in FP64 in
// every form: P inverts eigenvalues down to the 1e-11 cut, and an FP32
// product of a near-singular factor's P cancels to noise (negative scores
// included).
template <typename T, int CB>
__global__ void __launch_bounds__(kWideWarps * 32) normalize_wide_kernel(int R, int ldm,
                                                                         const int64_t* __restrict__ counters,
                                                                         const uint32_t* __restrict__ touched,
                                                                         const T* __restrict__ Uc,
                                                                         const double* __restrict__ sigma,
                                                                         const double* __restrict__ Pm,
                                                                         const int* __restrict__ degenerate,
                                                                         double* __restrict__ U,
                                                                         double* __restrict__ scores,
                                                                         double* __restrict__ scores_c) {
    constexpr int RP = 32 * CB;
    extern __shared__ __align__(16) unsigned char wide_dyn[];
    double* psm = reinterpret_cast<double*>(wide_dyn);  // [RP][RP] when Pm != null
    double* usm = psm + (Pm ? RP * RP : 0);             // [warps][RP]
    __shared__ double inv_sigma[kMaxRank];
    pdl_wait();
    pdl_trigger();
    // A zero column norm: the division of every row (as the reference does)
    // is left to scale_rows_if_degenerate; the FP64 rows are already in the
    // factor, the FP32 ones are copied there unscaled.
    const bool deg = *degenerate != 0;
    if (deg && !Uc) return;
    if (deg) Pm = nullptr;
    for (int c = threadIdx.x; c < R; c += blockDim.x) inv_sigma[c] = deg ? 1.0 : 1.0 / sigma[c];
    if (Pm)
        for (int e = threadIdx.x; e < RP * RP; e += blockDim.x) {
            const int a = e / RP, b = e % RP;
            psm[e] = (a < R && b < R) ? Pm[a * R + b] : 0.0;
        }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* u = usm + w * RP;
    const int64_t nt = counters[2];
    for (int64_t i = (int64_t)blockIdx.x * kWideWarps + w; i < nt; i += (int64_t)gridDim.x * kWideWarps) {
        const int64_t row = touched[i];
#pragma unroll
        for (int b = 0; b < CB; b++) {
            const int col = lane + 32 * b;
            double v = 0.0;
            if (col < R) {
                v = Uc ? (double)Uc[i * ldm + col] * inv_sigma[col] : U[row * R + col] * inv_sigma[col];
                U[row * R + col] = v;
            }
            u[col] = v;
        }
        if (Pm) {
            __syncwarp();
            double y = 0.0;
#pragma unroll
            for (int b = 0; b < CB; b++) {
                const int col = lane + 32 * b;
                double pu = 0.0;
                for (int a = 0; a < R; a++) pu = fma(psm[a * RP + col], u[a], pu);
                y = fma(u[col], pu, y);
            }
            y = warp_sum(y);
            if (lane == 0) {
                scores[row] = (double)y;
                scores_c[i] = (double)y;
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <typename T, int CB>
static int wide_mttkrp(Session& s, cudaStream_t st) {
    const bool f32 = std::is_same<T, float>::value;
    const int R = s.R;
    const int ldd = f32 ? f32_row_stride(R) : R;
    const int ldm = f32 ? f32_row_stride(R) : R;
    T* Mc = reinterpret_cast<T*>(s.Mc);
    T* cf = reinterpret_cast<T*>(s.carry_first);
    T* cl = reinterpret_cast<T*>(s.carry_last);
    const T* D = f32 ? reinterpret_cast<const T*>(s.Df) : reinterpret_cast<const T*>(s.D);
    const int hb = 152 * 8;
    // an ordinary launch: it follows the join with the side stream's design rows
    segreduce_wide_kernel<T, CB><<<hb, 256, 0, st>>>(R, ldd, ldm, s.counters, s.nnz, s.key_sorted,
                                                     f32 ? nullptr : s.pay_sorted, s.ex_j, (const double*)s.ex_val,
                                                     f32 ? s.pay64_sorted : nullptr, s.chunk_seg, D, Mc, cf, cl,
                                                     s.carry_row, s.carry_seg);
    count_launch();
    EXAFAC_CUDA_TRY(launch_dependent(segfix_kernel<T, kWideChunk, CB>, hb, 256, 0, st, R, ldm, s.counters, s.nnz,
                                     s.carry_row, s.carry_seg, s.seg_start, s.key_sorted, cf, cl, Mc));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

template <typename T, int CB>
static size_t wide_solve_smem() {
    return sizeof(T) * ((size_t)(32 * CB) * (32 * CB) + (size_t)kWideTileRows * (32 * CB + 4));
}

template <typename T, int CB>
static int wide_solve(Session& s, int n, cudaStream_t st) {
    const bool f32 = std::is_same<T, float>::value;
    const int ldm = f32 ? f32_row_stride(s.R) : s.R;
    const size_t smem = wide_solve_smem<T, CB>();
    EXAFAC_CUDA_TRY(
        cudaFuncSetAttribute(solve_gram_wide_kernel<T, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    EXAFAC_CUDA_TRY(launch_dependent_if(!s.dense[n], solve_gram_wide_kernel<T, CB>, kWideSolveBlocks,
                                        kWideWarps * 32, smem, st, s.R, ldm, s.counters, s.touched,
                                        reinterpret_cast<const T*>(s.Mc), s.dpinv, s.F.U[n],
                                        f32 ? reinterpret_cast<T*>(s.Uc) : nullptr, s.part));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

template <typename T, int CB>
static int wide_normalize(Session& s, int n, bool arls, cudaStream_t st) {
    const bool f32 = std::is_same<T, float>::value;
    const int R = s.R;
    EXAFAC_TRY(gram_reduce_to(s, kWideSolveBlocks, s.ugram, st));
    EXAFAC_TRY(sigma_and_gram(s, st));
    if (arls) EXAFAC_TRY(launch_pinv(R, s.ngram, s.upinv, 1e-11, s.vt, st));
    constexpr int RP = 32 * CB;
    const size_t smem = sizeof(double) * ((arls ? (size_t)RP * RP : 0) + (size_t)kWideWarps * RP);
    EXAFAC_CUDA_TRY(
        cudaFuncSetAttribute(normalize_wide_kernel<T, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    normalize_wide_kernel<T, CB><<<152 * 4, kWideWarps * 32, smem, st>>>(
        R, f32 ? f32_row_stride(R) : R, s.counters, s.touched, f32 ? reinterpret_cast<const T*>(s.Uc) : nullptr,
        s.F.sigma, arls ? s.upinv : nullptr, reinterpret_cast<int*>(s.counters + 6), s.F.U[n],
        arls ? s.scores[n] : nullptr, s.scores_c);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return scale_rows_if_degenerate(s, n, st);
}

template <typename T>
static int wide_step(Session& s, int n, cudaStream_t st, cudaEvent_t before_solve) {
    const int CB = (s.R + 31) / 32;
    switch (CB) {
        case 2: EXAFAC_TRY((wide_mttkrp<T, 2>(s, st))); break;
        case 3: EXAFAC_TRY((wide_mttkrp<T, 3>(s, st))); break;
        default: EXAFAC_TRY((wide_mttkrp<T, 4>(s, st))); break;
    }
    EXAFAC_TRY(clear_dense_factor(s, n, st));  // a never-updated factor is cleared before the writes
    if (before_solve) EXAFAC_CUDA_TRY(cudaStreamWaitEvent(st, before_solve, 0));
    switch (CB) {
        case 2: return wide_solve<T, 2>(s, n, st);
        case 3: return wide_solve<T, 3>(s, n, st);
        default: return wide_solve<T, 4>(s, n, st);
    }
}

template <typename T>
static int wide_norm(Session& s, int n, bool arls, cudaStream_t st) {
    const int CB = (s.R + 31) / 32;
    switch (CB) {
        case 2: return wide_normalize<T, 2>(s, n, arls, st);
        case 3: return wide_normalize<T, 3>(s, n, arls, st);
        default: return wide_normalize<T, 4>(s, n, arls, st);
    }
}

int mttkrp_solve_wide(Session& s, int n, cudaStream_t st, cudaEvent_t before_solve) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) return wide_step<double>(s, n, st, before_solve);
    return wide_step<float>(s, n, st, before_solve);
}

int normalize_wide(Session& s, int n, bool arls, cudaStream_t st) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) return wide_norm<double>(s, n, arls, st);
    return wide_norm<float>(s, n, arls, st);
}

}  // namespace exafac
