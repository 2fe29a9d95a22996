// Sampled MTTKRP and post-processing, load-balanced (R <= 32 path):
//
//   expand   hits in sample order: owner sample by one restricted binary search
//            per warp chunk; counts hits per output row
//   scatter  hits grouped by output row (counting sort)
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

constexpr int kExpandChunk = 256;  // hits per warp chunk in the expansion
constexpr int kSegChunk = 128;     // hits per warp chunk in the segmented reduction

static int grid_capped(int64_t work, int threads, int64_t cap = 152 * 16) {
    int64_t b = ceil_div(work, threads);
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

__device__ __forceinline__ int64_t owner_in(const int64_t* __restrict__ f_off, int64_t lo, int64_t hi, int64_t h) {
    // last j in [lo, hi) with f_off[j] <= h (f_off[lo] <= h guaranteed)
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (f_off[mid] <= h) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void hit_expand_kernel(const int64_t* __restrict__ counters, int64_t cap, const int64_t* __restrict__ f_off,
                                  const uint32_t* __restrict__ f_start, const uint32_t* __restrict__ rows_n,
                                  const double* __restrict__ vals_n, uint32_t* __restrict__ ex_row,
                                  uint32_t* __restrict__ ex_j, double* __restrict__ ex_val,
                                  uint32_t* __restrict__ rowcnt, DeviceStatus* status) {
    const int64_t ju = counters[0];
    int64_t H = counters[1];
    if (H > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) report(status, EXAFAC_ERR_DEVICE, 4, H, cap);
        H = cap;
    }
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c * kExpandChunk < H; c += nwarps) {
        const int64_t h0 = c * kExpandChunk;
        const int64_t h1 = min(H, h0 + kExpandChunk);
        // Owners of the chunk's first and last hits bound every owner in it.
        int64_t jlo = 0, jhi = 0;
        if (lane == 0) jlo = owner_in(f_off, 0, ju, h0);
        if (lane == 1) jhi = owner_in(f_off, 0, ju, h1 - 1) + 1;
        jlo = __shfl_sync(0xffffffffu, jlo, 0);
        jhi = __shfl_sync(0xffffffffu, jhi, 1);
        for (int64_t h = h0 + lane; h < h1; h += 32) {
            const int64_t j = owner_in(f_off, jlo, jhi, h);
            const int64_t p = (int64_t)f_start[j] + (h - f_off[j]);
            const uint32_t row = rows_n[p];
            ex_row[h] = row;
            ex_j[h] = (uint32_t)j;
            ex_val[h] = vals_n[p];
            atomicAdd(&rowcnt[row], 1u);
        }
    }
}

__global__ void hit_group_kernel(const int64_t* __restrict__ counters, int64_t cap, const uint32_t* __restrict__ ex_row,
                                 const uint32_t* __restrict__ ex_j, const double* __restrict__ ex_val,
                                 const int64_t* __restrict__ rowoff, uint32_t* __restrict__ rowfill,
                                 uint32_t* __restrict__ hit_row, uint32_t* __restrict__ hit_j,
                                 double* __restrict__ hit_val) {
    const int64_t H = min(counters[1], cap);
    for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < H; h += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t row = ex_row[h];
        const int64_t dst = rowoff[row] + atomicAdd(&rowfill[row], 1u);
        hit_row[dst] = row;
        hit_j[dst] = ex_j[h];
        hit_val[dst] = ex_val[h];
    }
}

// Segmented reduction over row-grouped hits, lane = column (R <= 32).
// Mc[i] (i = compact index of the touched row = pos[row]) receives rows that
// lie inside one chunk; crossing rows leave carries:
//   carry_first[c]: the chunk's first row when it started in an earlier chunk
//   carry_last[c]:  the chunk's last row when it continues in a later chunk
template <typename TD, typename TA>
__global__ void segreduce_kernel(int R, const int64_t* __restrict__ counters, int64_t cap,
                                 const uint32_t* __restrict__ hit_row, const uint32_t* __restrict__ hit_j,
                                 const double* __restrict__ hit_val, const int64_t* __restrict__ rowoff,
                                 const uint32_t* __restrict__ rowcnt, const int64_t* __restrict__ pos,
                                 const TD* __restrict__ D, TA* __restrict__ Mc, TA* __restrict__ carry_first,
                                 TA* __restrict__ carry_last) {
    const int64_t H = min(counters[1], cap);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c * kSegChunk < H; c += nwarps) {
        const int64_t cs = c * kSegChunk;
        const int64_t ce = min(H, cs + kSegChunk);
        int64_t h = cs;
        while (h < ce) {
            const uint32_t row = hit_row[h];
            const int64_t rs = rowoff[row], re = rs + rowcnt[row];
            const int64_t e = min(re, ce);
            TA acc = 0;
            if (lane < R) {
                for (int64_t p = h; p < e; p++) acc += (TA)D[(int64_t)hit_j[p] * R + lane] * (TA)hit_val[p];
            }
            if (lane < R) {
                if (rs >= cs && re <= ce) Mc[pos[row] * R + lane] = acc;
                else if (rs < cs) carry_first[c * R + lane] = acc;
                else carry_last[c * R + lane] = acc;
            }
            h = e;
        }
    }
}

// Crossing rows: sum their carries in chunk order.  Warp per touched row;
// rows inside one chunk are skipped.
template <typename TA>
__global__ void segfix_kernel(int R, const int64_t* __restrict__ counters, const uint32_t* __restrict__ touched,
                              const int64_t* __restrict__ rowoff, const uint32_t* __restrict__ rowcnt,
                              const TA* __restrict__ carry_first, const TA* __restrict__ carry_last,
                              TA* __restrict__ Mc) {
    const int64_t nt = counters[2];
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < nt; i += nwarps) {
        const uint32_t row = touched[i];
        const int64_t rs = rowoff[row], re = rs + rowcnt[row];
        const int64_t c0 = rs / kSegChunk, c1 = (re - 1) / kSegChunk;
        if (c0 == c1 || lane >= R) continue;
        TA acc = carry_last[c0 * R + lane];
        for (int64_t c = c0 + 1; c <= c1; c++) acc += carry_first[c * R + lane];
        Mc[i * R + lane] = acc;
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
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < R) m[k] = Mc[i * R + k];
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
int mttkrp_rows_balanced(Session& s, int n, cudaStream_t st) {
    const Lookup& L = s.look[n];
    const int64_t I = s.dims[n];
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.rowcnt, 0, sizeof(uint32_t) * I, st));
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.rowfill, 0, sizeof(uint32_t) * I, st));
    const int hb = 152 * 8;
    hit_expand_kernel<<<hb, 256, 0, st>>>(s.counters, s.nnz, s.f_off, s.f_start, L.rows, L.vals, s.ex_row, s.ex_j,
                                          s.ex_val, s.rowcnt, s.status);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    EXAFAC_TRY(scan_exclusive_u32_to_i64(s.rowcnt, s.rowoff, I, s.counters + 3, s.scan_sc, st));
    EXAFAC_TRY(touched_rows(s, I, st));
    hit_group_kernel<<<hb, 256, 0, st>>>(s.counters, s.nnz, s.ex_row, s.ex_j, s.ex_val, s.rowoff, s.rowfill,
                                         s.hit_row, s.hit_j, s.hit_val);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

constexpr int kSolveBlocks = 152 * 2;

template <typename TA>
static int segmented_mttkrp(Session& s, cudaStream_t st) {
    const int R = s.R;
    const int hb = 152 * 8;
    TA* Mc = reinterpret_cast<TA*>(s.Mc);
    TA* cf = reinterpret_cast<TA*>(s.carry_first);
    TA* cl = reinterpret_cast<TA*>(s.carry_last);
    if (std::is_same<TA, double>::value)
        segreduce_kernel<double, double><<<hb, 256, 0, st>>>(R, s.counters, s.nnz, s.hit_row, s.hit_j, s.hit_val,
                                                             s.rowoff, s.rowcnt, s.pos, (const double*)s.D,
                                                             (double*)Mc, (double*)cf, (double*)cl);
    else
        segreduce_kernel<float, float><<<hb, 256, 0, st>>>(R, s.counters, s.nnz, s.hit_row, s.hit_j, s.hit_val,
                                                           s.rowoff, s.rowcnt, s.pos, (const float*)s.Df, (float*)Mc,
                                                           (float*)cf, (float*)cl);
    count_launch();
    segfix_kernel<TA><<<hb, 256, 0, st>>>(R, s.counters, s.touched, s.rowoff, s.rowcnt, cf, cl, Mc);
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
    return solve_typed<float>(s, n, st);
}

int normalize_balanced(Session& s, int n, bool arls, cudaStream_t st) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) return normalize_typed<double>(s, n, arls, st);
    return normalize_typed<float>(s, n, arls, st);
}

__global__ void scatter_rows_kernel(int R, const int64_t* __restrict__ counters, const uint32_t* __restrict__ touched,
                                    const double* __restrict__ Mc, double* __restrict__ out) {
    const int64_t nt = counters[2];
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nt * R; e += (int64_t)gridDim.x * blockDim.x)
        out[(int64_t)touched[e / R] * R + e % R] = Mc[e];
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
