// Kernels of one sampled-ALS step after the draw (accumulator_stationary.hpp:
// 173-294 at one rank): deduplication, design rows + Gram, fiber lookup,
// sampled MTTKRP + R x R solve for R > 32, column renormalisation; plus the
// exact fit.
#include <cuda_bf16.h>

#include "dense.cuh"
#include "engine.cuh"
#include "mma.cuh"
#include "prims.cuh"

namespace exafac {

constexpr int kGramRows = 32;  // rows per block in the Gram partial kernels


static FactorPtrs factor_ptrs(const Session& s) {
    FactorPtrs f;
    for (int k = 0; k < kMaxModes; k++) f.U[k] = k < s.N ? s.F.U[k] : nullptr;
    return f;
}

static int grid_cap(int64_t work, int threads, int64_t cap = 152 * 16) {
    int64_t b = ceil_div(work, threads);
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

// ---------------------------------------------------------------------------
// Deduplication (deduplicate_design_matrix, als_optimizer.hpp:130-206).
// Unique rows are identified by a hash table keyed on the packed coordinates
// of the modes != n; each unique row is represented by its first occurrence,
// so the output order is the order of first occurrence.  Weight = the
// representative's weight times the multiplicity.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool keys_equal(Key128 a, Key128 b) { return a.lo == b.lo && a.hi == b.hi; }

// Each sample's key is packed once and published (dkey[j], then a fence)
// before the sample claims a slot, so a thread that meets the slot's owner
// compares against the owner's stored key instead of re-packing it.
__global__ void dedup_insert_kernel(KeySpec spec, int64_t J, const uint32_t* __restrict__ samples, int64_t mask,
                                    int32_t* owner, int32_t* minj, int32_t* count, int32_t* __restrict__ slot_of,
                                    Key128* dkey) {
    pdl_trigger();
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J) return;
    const Key128 key = pack_key(spec, samples + j * spec.N);
    dkey[j] = key;
    __threadfence();
    int64_t h = (int64_t)(hash_key(key) & (uint64_t)mask);
    for (int64_t probe = 0; probe <= mask; probe++) {
        int32_t o = atomicCAS(&owner[h], -1, (int32_t)j);
        if (o == -1) break;
        const volatile uint64_t* po = reinterpret_cast<const volatile uint64_t*>(&dkey[o]);
        Key128 ko;
        ko.lo = po[offsetof(Key128, lo) / 8];
        ko.hi = po[offsetof(Key128, hi) / 8];
        if (keys_equal(ko, key)) break;
        h = (h + 1) & mask;
    }
    atomicMin(&minj[h], (int32_t)j);
    atomicAdd(&count[h], 1);
    slot_of[j] = (int32_t)h;
}

// The representatives (first occurrences) in order, in two passes over tiles
// of kDedupTile samples (thread t holds samples 4t .. 4t + 3 of its tile):
// dedup_count_kernel counts each tile's representatives; dedup_place_kernel
// adds the counts of the tiles before its own (at most J / kDedupTile of
// them), scans its tile and writes the representatives' coordinates and
// weight x multiplicity at their places, and block 0 writes J_u to
// counters[0].
constexpr int kDedupTile = 1024;

__device__ __forceinline__ uint32_t dedup_rep_bits(int64_t J, int64_t j0, const int32_t* __restrict__ minj,
                                                   const int32_t* __restrict__ slot_of) {
    uint32_t bits = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int64_t j = j0 + k;
        if (j < J && minj[slot_of[j]] == (int32_t)j) bits |= 1u << k;
    }
    return bits;
}

__global__ void __launch_bounds__(256) dedup_count_kernel(int64_t J, const int32_t* __restrict__ minj,
                                                          const int32_t* __restrict__ slot_of,
                                                          uint32_t* __restrict__ tile_count) {
    __shared__ uint32_t wsum[8];
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t j0 = (int64_t)blockIdx.x * kDedupTile + 4 * threadIdx.x;
    uint32_t c = (uint32_t)__popc(dedup_rep_bits(J, j0, minj, slot_of));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) wsum[w] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int ww = 0; ww < 8; ww++) t += wsum[ww];
        tile_count[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(256) dedup_place_kernel(int N, int64_t J, int64_t ntiles,
                                                          const uint32_t* __restrict__ tile_count,
                                                          const int32_t* __restrict__ minj,
                                                          const int32_t* __restrict__ slot_of,
                                                          const int32_t* __restrict__ count,
                                                          const uint32_t* __restrict__ samples,
                                                          const double* __restrict__ weights,
                                                          uint32_t* __restrict__ sd, double* __restrict__ wd,
                                                          int64_t* __restrict__ ju_out) {
    pdl_wait();
    pdl_trigger();
    __shared__ uint32_t wsum[8];
    __shared__ int64_t before_sh;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // representatives of the tiles before this one, and of all tiles (block 0)
    int64_t a = 0, all = 0;
    for (int64_t i = threadIdx.x; i < ntiles; i += blockDim.x) {
        const int64_t v = tile_count[i];
        all += v;
        if (i < (int64_t)blockIdx.x) a += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        all += __shfl_xor_sync(0xffffffffu, all, o);
    }
    __shared__ int64_t red_a[8], red_all[8];
    if (lane == 0) {
        red_a[w] = a;
        red_all[w] = all;
    }
    const int64_t j0 = (int64_t)blockIdx.x * kDedupTile + 4 * threadIdx.x;
    const uint32_t bits = dedup_rep_bits(J, j0, minj, slot_of);
    const uint32_t c = (uint32_t)__popc(bits);
    uint32_t inc = c;  // inclusive scan of the threads' counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t ta = 0, tall = 0;
        for (int ww = 0; ww < 8; ww++) {
            ta += red_a[ww];
            tall += red_all[ww];
        }
        before_sh = ta;
        if (blockIdx.x == 0) *ju_out = tall;
    }
    __syncthreads();
    int64_t p = before_sh + inc - c;
    for (int ww = 0; ww < w; ww++) p += wsum[ww];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!((bits >> k) & 1u)) continue;
        const int64_t j = j0 + k;
        for (int m = 0; m < N; m++) sd[p * N + m] = samples[j * N + m];
        wd[p] = weights[j] * (double)count[slot_of[j]];
        p++;
    }
}

int dedup(Session& s, int n, int64_t J, cudaStream_t st) {
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.d_owner, 0xff, sizeof(int32_t) * s.dtab, st));
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.d_minj, 0x7f, sizeof(int32_t) * s.dtab, st));
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.d_count, 0, sizeof(int32_t) * s.dtab, st));
    const unsigned blocks = (unsigned)ceil_div(J, 256);
    dedup_insert_kernel<<<blocks, 256, 0, st>>>(s.look[n].spec, J, s.samples, s.dtab - 1, s.d_owner, s.d_minj,
                                                s.d_count, s.slot_of, s.dkey); count_launch();
    const int64_t ntiles = ceil_div(J, kDedupTile);
    EXAFAC_CUDA_TRY(launch_dependent(dedup_count_kernel, (unsigned)ntiles, 256, 0, st, J, s.d_minj, s.slot_of, s.flags));
    count_launch();
    EXAFAC_CUDA_TRY(launch_dependent(dedup_place_kernel, (unsigned)ntiles, 256, 0, st, s.N, J, ntiles, s.flags,
                                     s.d_minj, s.slot_of, s.d_count, s.samples, s.weights, s.sd, s.wd,
                                     s.counters + 0));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// ---------------------------------------------------------------------------
// Gram partials and their deterministic reduction.
// ---------------------------------------------------------------------------
__global__ void gram_reduce_kernel(const double* __restrict__ part, int64_t nblk, int R, double* __restrict__ out) {
    __shared__ double red[256];
    pdl_wait();
    pdl_trigger();
    const int P = packed_size(R);
    const int e = blockIdx.x;
    if (e >= P) return;
    double acc = 0.0;
    for (int64_t b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[b * P + e];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int a = 0, rem = e;
        while (rem >= R - a) {
            rem -= R - a;
            a++;
        }
        int b = a + rem;
        out[a * R + b] = red[0];
        out[b * R + a] = red[0];
    }
}

// Gram of rows of A (all `rows`, or the first *count_dev entries of rowlist).
__global__ void gram_partial_kernel(int R, const double* __restrict__ A, int64_t rows, const uint32_t* __restrict__ list,
                                    const int64_t* __restrict__ count_dev, double* __restrict__ part) {
    extern __shared__ double sm[];
    const int P = packed_size(R);
    const int64_t cnt = list ? *count_dev : rows;
    const int64_t base = (int64_t)blockIdx.x * kGramRows;
    for (int e = threadIdx.x; e < kGramRows * R; e += blockDim.x) {
        int lr = e / R, c = e % R;
        int64_t i = base + lr;
        double v = 0.0;
        if (i < cnt) {
            int64_t r = list ? (int64_t)list[i] : i;
            v = A[r * R + c];
        }
        sm[lr * R + c] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        int a = 0, rem = e;
        while (rem >= R - a) {
            rem -= R - a;
            a++;
        }
        int b = a + rem;
        double acc = 0.0;
        for (int lr = 0; lr < kGramRows; lr++) acc = fma(sm[lr * R + a], sm[lr * R + b], acc);
        part[(int64_t)blockIdx.x * P + e] = acc;
    }
}

int gram_rows(Session& s, const double* A, int64_t rows, const uint32_t* rowlist, const int64_t* count_dev,
              double* out_full, cudaStream_t st) {
    const int R = s.R;
    int64_t nblk = std::max<int64_t>(1, ceil_div(rows, kGramRows));
    if (nblk > s.part_rows) {
        set_error("gram_rows: partial buffer too small");
        return EXAFAC_ERR_WORKSPACE;
    }
    gram_partial_kernel<<<(unsigned)nblk, 128, sizeof(double) * kGramRows * R, st>>>(R, A, rows, rowlist, count_dev,
                                                                                     s.part); count_launch();
    gram_reduce_kernel<<<packed_size(R), 256, 0, st>>>(s.part, nblk, R, out_full); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// ---------------------------------------------------------------------------
// Design rows (accumulator_stationary.hpp:212-249): D_j = prod_{k!=n}
// U_k[s_jk] (mode order, from 1.0), D_j *= sqrt(w_j); Gram of these rows;
// the rows used by the MTTKRP are scaled by sqrt(w_j) once more.
// ---------------------------------------------------------------------------
__global__ void design_kernel(int N, int n, int R, const int64_t* __restrict__ ju_dev, const uint32_t* __restrict__ sd,
                              const double* __restrict__ wd, FactorPtrs f, double* __restrict__ D,
                              double* __restrict__ part) {
    extern __shared__ double sm[];
    const int P = packed_size(R);
    const int64_t ju = *ju_dev;
    const int64_t base = (int64_t)blockIdx.x * kGramRows;
    for (int e = threadIdx.x; e < kGramRows * R; e += blockDim.x) {
        int lr = e / R, c = e % R;
        int64_t j = base + lr;
        double v = 0.0;
        if (j < ju) {
            double d = 1.0;
            for (int k = 0; k < N; k++) {
                if (k == n) continue;
                d *= f.U[k][(int64_t)sd[j * N + k] * R + c];
            }
            const double sw = sqrt(wd[j]);
            d *= sw;
            v = d;
            D[j * R + c] = d * sw;
        }
        sm[lr * R + c] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        int a = 0, rem = e;
        while (rem >= R - a) {
            rem -= R - a;
            a++;
        }
        int b = a + rem;
        double acc = 0.0;
        for (int lr = 0; lr < kGramRows; lr++) acc = fma(sm[lr * R + a], sm[lr * R + b], acc);
        part[(int64_t)blockIdx.x * P + e] = acc;
    }
}

// Mixed forms: the same design rows with FP32 row products, the MTTKRP
// operand D' kept in FP32, and the Gram of the sqrt(w)-scaled rows from
// inputs rounded to TF32 (10-bit mantissa, round to nearest) or BF16 (7-bit)
// on the tensor cores, accumulated in FP32 within a block of 32 rows and in
// FP64 across blocks.
__device__ __forceinline__ float round_bf16(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Tensor-core form.  A warp owns 32 design rows at a time:
//   * factor rows are gathered one per load instruction (lane = column),
//     32 rows in flight per mode, rounded to FP32 in integer arithmetic
//     (narrow_f64, off the FP64 pipe) and multiplied in FP32;
//   * D'_j = d_j * w_j goes to Df (FP32, rows of 32 floats: one 128-byte
//     line per row for the gathers of the segmented reduction,
//     zero padded), the Gram input round(d_j sqrt(w_j))
//     to a shared tile T (32 rows x kDStride, zero padded);
//   * the tile's Gram T^T T comes from mma.sync m16n8k8 TF32 instructions with
//     FP32 accumulation (only the 16 x 8 blocks on or below the diagonal),
//     added to compensated FP32 sums (hi + lo) after every 32-row tile, and
//     to FP64 once per warp at the end.  BF16-rounded inputs
//     are exact in TF32, so the same instruction serves both roundings.
// The block's warps are summed in warp order into part[block] (packed).
constexpr int kDesignWarps = 8;
constexpr int kDStride = 40;  // floats per tile row: fragment loads hit 32 distinct banks
constexpr int kDesignBlocks = 152 * 2;


template <int kRound>  // 1: TF32, 2: BF16
__global__ void __launch_bounds__(kDesignWarps * 32) design_mma_kernel(int N, int n, int R,
                                                                       const int64_t* __restrict__ ju_dev,
                                                                       const uint32_t* __restrict__ sd,
                                                                       const double* __restrict__ wd, FactorPtrs f,
                                                                       float* __restrict__ Df,
                                                                       double* __restrict__ part) {
    // the warps' tiles; at the end the per-warp Gram sums (kDesignWarps x P doubles)
    __shared__ __align__(16) float tile[kDesignWarps][32][kDStride];
    __shared__ uint32_t sidx[kDesignWarps][kMaxModes][32];  // the tile's sample indices, all modes
    static_assert(sizeof(tile) >= sizeof(float2) * kDesignWarps * (32 * 33 / 2), "slab does not fit");
    // lower-triangle (m-tile, n-tile) pairs of the 32 x 32 Gram: 16-row m-tiles, 8-column n-tiles
    constexpr int kPairs = 6;
    constexpr int kMt[kPairs] = {0, 0, 1, 1, 1, 1};
    constexpr int kNt[kPairs] = {0, 1, 0, 1, 2, 3};
    const int P = R * (R + 1) / 2;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    float ghi[kPairs][4], glo[kPairs][4];  // compensated sums over the warp's tiles
#pragma unroll
    for (int p = 0; p < kPairs; p++)
#pragma unroll
        for (int i = 0; i < 4; i++) ghi[p][i] = glo[p][i] = 0.0f;
    float (*t)[kDStride] = tile[w];
    const int RS = (R + 3) & ~3;  // Df row length written (zero padded); the row stride is 32
    const int64_t ju = *ju_dev;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < ju; base += nwarps * 32) {
        const int nrow = (int)min((int64_t)32, ju - base);
        float prod[32];
#pragma unroll
        for (int r = 0; r < 32; r++) prod[r] = 1.0f;
        // every mode's indices in one round of loads, before the first gather
        for (int k = 0; k < N; k++) sidx[w][k][lane] = lane < nrow ? sd[(base + lane) * N + k] : 0u;
        __syncwarp();
        for (int k = 0; k < N; k++) {
            if (k == n) continue;
            const uint32_t myidx = sidx[w][k][lane];
            const double* Uk = f.U[k];
#pragma unroll
            for (int r = 0; r < 32; r++) {
                const int64_t i = __shfl_sync(0xffffffffu, myidx, r);
                if (r < nrow && lane < R) prod[r] *= narrow_f64(Uk[i * R + lane]);
            }
        }
        const float myw = lane < nrow ? narrow_f64(wd[base + lane]) : 0.0f, mysw = sqrtf(myw);
#pragma unroll
        for (int r = 0; r < 32; r++) {
            const float wr = __shfl_sync(0xffffffffu, myw, r), swr = __shfl_sync(0xffffffffu, mysw, r);
            float v = 0.0f;
            if (r < nrow && lane < R) {
                const float x = prod[r] * swr;
                v = kRound == 1 ? round_tf32(x) : round_bf16(x);
            }
            if (r < nrow && lane < RS) Df[(base + r) * 32 + lane] = lane < R ? prod[r] * wr : 0.0f;
            t[r][lane] = v;  // lanes >= R and rows >= nrow: zero
        }
        __syncwarp();
        float c[kPairs][4];
#pragma unroll
        for (int p = 0; p < kPairs; p++)
#pragma unroll
            for (int i = 0; i < 4; i++) c[p][i] = 0.0f;
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {
            const int k0 = ks * 8 + tig;
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {  // A = T^T: A[m][k] = T[k][m]
                af[mt][0] = __float_as_uint(t[k0][16 * mt + gid]);
                af[mt][1] = __float_as_uint(t[k0][16 * mt + gid + 8]);
                af[mt][2] = __float_as_uint(t[k0 + 4][16 * mt + gid]);
                af[mt][3] = __float_as_uint(t[k0 + 4][16 * mt + gid + 8]);
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {  // B = T: B[k][n] = T[k][n]
                bf[nt][0] = __float_as_uint(t[k0][8 * nt + gid]);
                bf[nt][1] = __float_as_uint(t[k0 + 4][8 * nt + gid]);
            }
#pragma unroll
            for (int p = 0; p < kPairs; p++) mma_tf32_16x8x8(c[p], af[kMt[p]], bf[kNt[p]]);
        }
#pragma unroll
        for (int p = 0; p < kPairs; p++)
#pragma unroll
            for (int i = 0; i < 4; i++) two_sum_acc(ghi[p][i], glo[p][i], c[p][i]);
        __syncwarp();
    }
    // Block sum in warp order: every warp leaves its (hi, lo) sums in its row
    // of the slab (each packed entry has exactly one owner lane per warp),
    // then a thread per entry adds the rows in order, still compensated, and
    // widens once (no FP64 arithmetic but the final hi + lo).
    __syncthreads();
    float2* slab = reinterpret_cast<float2*>(&tile[0][0][0]);
#pragma unroll
    for (int p = 0; p < kPairs; p++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int row = 16 * kMt[p] + gid + 8 * (i >> 1);
            const int col = 8 * kNt[p] + 2 * tig + (i & 1);
            if (row < R && col <= row) slab[w * P + packed_index(R, col, row)] = make_float2(ghi[p][i], glo[p][i]);
        }
    __syncthreads();
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        float hi = 0.0f, lo = 0.0f;
#pragma unroll
        for (int ww = 0; ww < kDesignWarps; ww++) {
            const float2 v = slab[ww * P + e];
            two_sum_acc(hi, lo, v.x);
            lo += v.y;
        }
        part[(int64_t)blockIdx.x * P + e] = widen_f32(hi) + widen_f32(lo);
    }
}

// R > 32 (padded to RP = 64 or 128): the block's 8 warps share one 32-row
// tile (warp w builds rows 4w..4w+3, FP64 row products, D' = d w rounded to
// FP32 for the FP32 MTTKRP), and split the lower-triangle 16 x 8 MMA blocks of the
// RP x RP Gram between them; each Gram entry has one owner, so the block sum
// needs no ordering.
template <int kRound, int RP>
__global__ void __launch_bounds__(kDesignWarps * 32) design_mma_wide_kernel(int N, int n, int R,
                                                                            const int64_t* __restrict__ ju_dev,
                                                                            const uint32_t* __restrict__ sd,
                                                                            const double* __restrict__ wd,
                                                                            FactorPtrs f, float* __restrict__ Df,
                                                                            double* __restrict__ part) {
    constexpr int kStride = RP + 8;  // row stride mod 32 == 8: conflict-free fragment loads
    const int ldf = f32_row_stride(R);  // FP32 design rows for the FP32 MTTKRP
    constexpr int kMT = RP / 16;
    constexpr int kPairs = kMT * (kMT + 1);  // m-tile mt pairs with n-tiles 0 .. 2 mt + 1
    constexpr int kPerWarp = (kPairs + kDesignWarps - 1) / kDesignWarps;
    constexpr int kCB = RP / 32;
    extern __shared__ __align__(16) unsigned char dyn[];
    float (*t)[kStride] = reinterpret_cast<float (*)[kStride]>(dyn);
    double* red = reinterpret_cast<double*>(dyn + sizeof(float) * 32 * kStride);
    const int P = R * (R + 1) / 2;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    for (int e = threadIdx.x; e < P; e += blockDim.x) red[e] = 0.0;
    int pm[kPerWarp], pn[kPerWarp];
#pragma unroll
    for (int q = 0; q < kPerWarp; q++) {
        const int p = w + kDesignWarps * q;
        int mt = 0, rem = p;
        while (mt < kMT && rem >= 2 * (mt + 1)) {
            rem -= 2 * (mt + 1);
            mt++;
        }
        pm[q] = p < kPairs ? mt : -1;
        pn[q] = rem;
    }
    double gacc[kPerWarp][4];
#pragma unroll
    for (int q = 0; q < kPerWarp; q++)
#pragma unroll
        for (int i = 0; i < 4; i++) gacc[q][i] = 0.0;
    __syncthreads();
    const int64_t ju = *ju_dev;
    for (int64_t base = (int64_t)blockIdx.x * 32; base < ju; base += (int64_t)gridDim.x * 32) {
        const int nrow = (int)min((int64_t)32, ju - base);
        // the sample indices of the warp's four rows for every mode (lane
        // l < 4 N: row l / N, mode l % N) and their weights, in one round of
        // loads before the first gather
        int64_t myi = 0;
        double myw = 0.0;
        if (lane < 4 * N) {
            const int rr = lane / N, k = lane - rr * N;
            if (4 * w + rr < nrow) myi = sd[(base + 4 * w + rr) * N + k];
        }
        if (lane < 4 && 4 * w + lane < nrow) myw = wd[base + 4 * w + lane];
        for (int rr = 0; rr < 4; rr++) {
            const int r = 4 * w + rr;
            const int64_t j = base + r;
            double d[kCB];
#pragma unroll
            for (int cb = 0; cb < kCB; cb++) d[cb] = 1.0;
            const double wj = __shfl_sync(0xffffffffu, myw, rr);
            if (r < nrow) {  // uniform over the warp
                // modes unrolled: the factor pointers stay in the parameter
                // bank and a row's gathers of every mode are independent
#pragma unroll
                for (int k = 0; k < kMaxModes; k++) {
                    if (k >= N || k == n) continue;
                    const int64_t i = __shfl_sync(0xffffffffu, myi, rr * N + k);
                    const double* ur = f.U[k] + i * R;
#pragma unroll
                    for (int cb = 0; cb < kCB; cb++) {
                        const int c = lane + 32 * cb;
                        if (c < R) d[cb] *= ur[c];
                    }
                }
            }
            const double sw = sqrt(r < nrow ? wj : 0.0);
#pragma unroll
            for (int cb = 0; cb < kCB; cb++) {
                const int c = lane + 32 * cb;
                float v = 0.0f;
                if (r < nrow && c < R) {
                    const double x = d[cb] * sw;
                    Df[j * ldf + c] = (float)(x * sw);
                    v = kRound == 1 ? round_tf32((float)x) : round_bf16((float)x);
                }
                t[r][c] = v;
            }
        }
        __syncthreads();
        float c[kPerWarp][4];
#pragma unroll
        for (int q = 0; q < kPerWarp; q++)
#pragma unroll
            for (int i = 0; i < 4; i++) c[q][i] = 0.0f;
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {
            const int k0 = ks * 8 + tig;
#pragma unroll
            for (int q = 0; q < kPerWarp; q++) {
                if (pm[q] < 0) continue;
                const int m0 = 16 * pm[q], n0 = 8 * pn[q];
                const uint32_t a[4] = {__float_as_uint(t[k0][m0 + gid]), __float_as_uint(t[k0][m0 + gid + 8]),
                                       __float_as_uint(t[k0 + 4][m0 + gid]), __float_as_uint(t[k0 + 4][m0 + gid + 8])};
                const uint32_t b[2] = {__float_as_uint(t[k0][n0 + gid]), __float_as_uint(t[k0 + 4][n0 + gid])};
                mma_tf32_16x8x8(c[q], a, b);
            }
        }
#pragma unroll
        for (int q = 0; q < kPerWarp; q++)
#pragma unroll
            for (int i = 0; i < 4; i++) gacc[q][i] += (double)c[q][i];
        __syncthreads();  // the next tile overwrites t
    }
#pragma unroll
    for (int q = 0; q < kPerWarp; q++) {
        if (pm[q] < 0) continue;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int row = 16 * pm[q] + gid + 8 * (i >> 1);
            const int col = 8 * pn[q] + 2 * tig + (i & 1);
            if (row < R && col <= row) red[packed_index(R, col, row)] = gacc[q][i];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < P; e += blockDim.x) part[(int64_t)blockIdx.x * P + e] = red[e];
}

template <int kRound, int RP>
static int launch_design_wide(Session& s, int n, cudaStream_t st) {
    const size_t smem = sizeof(float) * 32 * (RP + 8) + sizeof(double) * packed_size(RP);
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(design_mma_wide_kernel<kRound, RP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    design_mma_wide_kernel<kRound, RP><<<kDesignBlocks, kDesignWarps * 32, smem, st>>>(
        s.N, n, s.R, s.counters + 0, s.sd, s.wd, factor_ptrs(s), s.Df, s.part);
    count_launch();
    return EXAFAC_OK;
}

int design_gram(Session& s, int n, int64_t J, cudaStream_t st) {
    const int R = s.R;
    int64_t nblk = std::max<int64_t>(1, ceil_div(J, kGramRows));
    if (s.cfg.precision != EXAFAC_PREC_FP64) {
        const bool tf32 = s.cfg.precision == EXAFAC_PREC_TF32;
        if (R > 32) {  // FP32 design rows for the FP32 MTTKRP, tensor-core Gram
            int rc;
            if (R <= 64) rc = tf32 ? launch_design_wide<1, 64>(s, n, st) : launch_design_wide<2, 64>(s, n, st);
            else rc = tf32 ? launch_design_wide<1, 128>(s, n, st) : launch_design_wide<2, 128>(s, n, st);
            EXAFAC_TRY(rc);
            gram_reduce_kernel<<<packed_size(R), 256, 0, st>>>(s.part, kDesignBlocks, R, s.dgram); count_launch();
            EXAFAC_CHECK_LAUNCH();
            return EXAFAC_OK;
        }
        if (tf32)
            design_mma_kernel<1><<<kDesignBlocks, kDesignWarps * 32, 0, st>>>(s.N, n, R, s.counters + 0, s.sd, s.wd,
                                                                               factor_ptrs(s), s.Df, s.part);
        else
            design_mma_kernel<2><<<kDesignBlocks, kDesignWarps * 32, 0, st>>>(s.N, n, R, s.counters + 0, s.sd, s.wd,
                                                                               factor_ptrs(s), s.Df, s.part);
        count_launch();
        gram_reduce_kernel<<<packed_size(R), 256, 0, st>>>(s.part, kDesignBlocks, R, s.dgram); count_launch();
        EXAFAC_CHECK_LAUNCH();
        return EXAFAC_OK;
    }
    design_kernel<<<(unsigned)nblk, 128, sizeof(double) * kGramRows * R, st>>>(s.N, n, R, s.counters + 0, s.sd, s.wd,
                                                                               factor_ptrs(s), s.D, s.part); count_launch();
    gram_reduce_kernel<<<packed_size(R), 256, 0, st>>>(s.part, nblk, R, s.dgram); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// Phi = pseudo-inverse of the design Gram: compute_pinv_square
// (common.h:405-443, eigenvalue cut 1e-11); the mixed forms add one Newton
// step X <- X (2I - G X) on the FP32-accumulated Gram.
int design_pinv(Session& s, cudaStream_t st) {
    if (s.cfg.precision != EXAFAC_PREC_FP64) return launch_pinv_refined(s.R, s.dgram, s.dpinv, 1e-11, s.vt, st);
    return launch_pinv(s.R, s.dgram, s.dpinv, 1e-11, s.vt, st);
}

// ---------------------------------------------------------------------------
// Fiber lookup + counting sort of the hits by output row
// (csr_based_spmm lookup half and transpose, sort_lookup.hpp:279-345).
// ---------------------------------------------------------------------------
template <typename Slot>
__device__ __forceinline__ bool slot_match(const Slot& sl, Key128 k);
template <>
__device__ __forceinline__ bool slot_match<Slot1>(const Slot1& sl, Key128 k) {
    return sl.key == k.lo;
}
template <>
__device__ __forceinline__ bool slot_match<Slot2>(const Slot2& sl, Key128 k) {
    return sl.lo == k.lo && sl.hi == k.hi;
}

template <typename Slot>
__global__ void lookup_kernel(KeySpec spec, int64_t J, const int64_t* __restrict__ ju_dev,
                              const uint32_t* __restrict__ sd, const Slot* __restrict__ slots, int64_t mask,
                              uint32_t* __restrict__ f_start, uint32_t* __restrict__ f_len) {
    pdl_trigger();
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J) return;
    uint32_t start = 0, len = 0;
    if (j < *ju_dev) {
        const Key128 key = pack_key(spec, sd + j * spec.N);
        int64_t h = (int64_t)(hash_key(key) & (uint64_t)mask);
        for (int64_t probe = 0; probe <= mask; probe++) {
            const Slot sl = slots[h];
            if (sl.start == kEmpty) break;
            if (slot_match(sl, key)) {
                start = sl.start;
                len = sl.len;
                break;
            }
            h = (h + 1) & mask;
        }
    }
    f_start[j] = start;
    f_len[j] = len;
}


int lookup_fibers(Session& s, int n, int64_t J, cudaStream_t st) {
    const Lookup& L = s.look[n];
    const unsigned blocks = (unsigned)ceil_div(J, 256);
    count_launch();
    if (L.kw == 1)
        lookup_kernel<Slot1><<<blocks, 256, 0, st>>>(L.spec, J, s.counters + 0, s.sd, (const Slot1*)L.slots,
                                                    L.nslots - 1, s.f_start, s.f_len);
    else
        lookup_kernel<Slot2><<<blocks, 256, 0, st>>>(L.spec, J, s.counters + 0, s.sd, (const Slot2*)L.slots,
                                                    L.nslots - 1, s.f_start, s.f_len);
    EXAFAC_CHECK_LAUNCH();
    // H to counters[1]; counters[5] accumulates the hits of all steps
    EXAFAC_TRY(scan_exclusive_u32_to_i64(s.f_len, s.f_off, J, s.counters + 1, s.scan_sc, st, s.counters + 5));
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int lookup_hits(Session& s, int n, int64_t J, bool packed, cudaStream_t st) {
    EXAFAC_TRY(lookup_fibers(s, n, J, st));
    return hits_by_row(s, n, packed, st);
}

// ---------------------------------------------------------------------------
// Sampled MTTKRP + solve (csr_based_spmm scatter half sort_lookup.hpp:347-371,
// then parallel_dsymm accumulator_stationary.hpp:283-286): warp per touched
// row, M_r = sum over the row's hits of val * D'[j], U_r = M_r * Phi.
// ---------------------------------------------------------------------------
__global__ void spmm_solve_kernel(int R, const int64_t* __restrict__ counters, const uint32_t* __restrict__ touched,
                                  const int64_t* __restrict__ seg_start, const uint32_t* __restrict__ pay,
                                  const uint32_t* __restrict__ ex_j, const double* __restrict__ ex_val,
                                  const double* __restrict__ D, const double* __restrict__ Phi, double* __restrict__ U) {
    extern __shared__ double sm[];
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* phi = sm;
    double* msm = sm + R * R + w * R;
    if (Phi)
        for (int e = threadIdx.x; e < R * R; e += blockDim.x) phi[e] = Phi[e];
    __syncthreads();
    const int64_t nt = counters[2];
    for (int64_t i = (int64_t)blockIdx.x * warps + w; i < nt; i += (int64_t)gridDim.x * warps) {
        const int64_t r = touched[i];
        const int64_t beg = seg_start[i], end = seg_start[i + 1];
        for (int c = lane; c < R; c += 32) {
            double acc = 0.0;
            for (int64_t p = beg; p < end; p++) {
                const uint32_t h = pay[p];
                acc += D[(int64_t)ex_j[h] * R + c] * ex_val[h];
            }
            msm[c] = acc;
        }
        __syncwarp();
        for (int c = lane; c < R; c += 32) {
            double acc;
            if (Phi) {
                acc = 0.0;
                for (int k = 0; k < R; k++) acc = fma(msm[k], phi[k * R + c], acc);
            } else {
                acc = msm[c];
            }
            U[r * R + c] = acc;
        }
        __syncwarp();
    }
}

int spmm_solve_into(Session& s, int n, const double* Phi, double* out, cudaStream_t st) {
    const int R = s.R;
    const int warps = 8;
    size_t smem = sizeof(double) * ((size_t)R * R + warps * R);
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(spmm_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    spmm_solve_kernel<<<grid_cap(s.dims[n], warps * 32), warps * 32, smem, st>>>(
        R, s.counters, s.touched, s.seg_start, s.pay_sorted, s.ex_j, s.ex_val, s.D, Phi, out); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int spmm_solve(Session& s, int n, cudaStream_t st) { return spmm_solve_into(s, n, s.dpinv, s.F.U[n], st); }

// ---------------------------------------------------------------------------
// Column renormalisation (DistMat1D::renormalize_columns, distmat.hpp:85-138).
// ---------------------------------------------------------------------------
__global__ void sigma_kernel(int R, const double* __restrict__ ugram, double* __restrict__ sigma,
                             double* __restrict__ ngram, int* __restrict__ degenerate) {
    __shared__ double sg[kMaxRank];
    __shared__ int deg;
    if (threadIdx.x == 0) deg = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < R; c += blockDim.x) {
        double v = sqrt(ugram[c * R + c]);
        sg[c] = v;
        sigma[c] = v;
        if (!(v > 0.0)) deg = 1;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) ngram[e] = ugram[e] / (sg[e / R] * sg[e % R]);
    if (threadIdx.x == 0) *degenerate = deg;
}

__global__ void scale_rows_kernel(int R, int64_t I, const uint32_t* __restrict__ list, const int64_t* __restrict__ cnt_dev,
                                  const double* __restrict__ sigma, const int* __restrict__ degenerate,
                                  double* __restrict__ U, int only_degenerate) {
    pdl_wait();
    pdl_trigger();
    if (only_degenerate && *degenerate == 0) return;
    const bool all = *degenerate != 0 || list == nullptr;
    const int64_t rows = all ? I : *cnt_dev;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < rows * R; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e / R;
        int c = (int)(e % R);
        int64_t r = all ? i : (int64_t)list[i];
        U[r * R + c] /= sigma[c];
    }
}

int normalize_factor(Session& s, int n, bool all_rows, cudaStream_t st) {
    const int R = s.R;
    const uint32_t* list = all_rows ? nullptr : s.touched;
    EXAFAC_TRY(gram_rows(s, s.F.U[n], s.dims[n], list, s.counters + 2, s.ugram, st));
    int* deg = reinterpret_cast<int*>(s.counters + 6);
    sigma_kernel<<<1, 256, 0, st>>>(R, s.ugram, s.F.sigma, s.ngram, deg); count_launch();
    scale_rows_kernel<<<grid_cap(s.dims[n] * R, 256), 256, 0, st>>>(R, s.dims[n], list, s.counters + 2, s.F.sigma,
                                                                     deg, s.F.U[n], 0); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int gram_reduce_to(Session& s, int64_t nblk, double* out, cudaStream_t st) {
    gram_reduce_kernel<<<packed_size(s.R), 256, 0, st>>>(s.part, nblk, s.R, out); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int sigma_and_gram(Session& s, cudaStream_t st) {
    sigma_kernel<<<1, 256, 0, st>>>(s.R, s.ugram, s.F.sigma, s.ngram, reinterpret_cast<int*>(s.counters + 6));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// The reference divides every row by the column norms; when a norm is zero
// the rows outside the touched list turn into NaN there too.  Exits at once
// unless a norm is zero.
int scale_rows_if_degenerate(Session& s, int n, cudaStream_t st) {
    EXAFAC_CUDA_TRY(launch_dependent(scale_rows_kernel, 152 * 4, 256, 0, st, s.R, s.dims[n], nullptr, s.counters + 2,
                                     s.F.sigma, reinterpret_cast<int*>(s.counters + 6), s.F.U[n], 1));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// The step's touched rows become mode n's nonzero-row list (nzrows[n],
// nzcount[n]): only the counters[2] listed entries are copied.
__global__ void keep_touched_kernel(const int64_t* __restrict__ counters, const uint32_t* __restrict__ touched,
                                    uint32_t* __restrict__ list, int64_t* __restrict__ count) {
    pdl_wait();
    pdl_trigger();
    const int64_t T = counters[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = T;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x)
        list[i] = touched[i];
}

int keep_touched(Session& s, int n, cudaStream_t st) {
    // follows the CDF build's last kernel (CP-ARLS-LEV)
    EXAFAC_CUDA_TRY(launch_dependent_if(s.cfg.sampler == EXAFAC_SAMPLER_CP_ARLS_LEV, keep_touched_kernel, 152 * 4, 256,
                                        0, st, s.counters, s.touched, s.nzrows[n], s.nzcount + n));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// Warp per 32 listed rows: indices loaded together, then one row per store
// instruction (lane = column).
// Rows listed in `keep` (a bitmap over the rows) are skipped: they are
// rewritten by the current update.
__global__ void zero_rows_kernel(int R, const uint32_t* __restrict__ list, const int64_t* __restrict__ cnt_dev,
                                 const uint32_t* __restrict__ keep, double* __restrict__ U,
                                 double* __restrict__ scores) {
    const int64_t cnt = *cnt_dev;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < cnt; base += nwarps * 32) {
        const int n = (int)min((int64_t)32, cnt - base);
        uint32_t myrow = lane < n ? list[base + lane] : 0u;
        bool clear = lane < n && !(keep && ((keep[myrow >> 5] >> (myrow & 31)) & 1u));
        if (scores && clear) scores[myrow] = 0.0;
        unsigned todo = __ballot_sync(0xffffffffu, clear);
        while (todo) {
            const int r = __ffs(todo) - 1;
            todo &= todo - 1;
            const int64_t row = __shfl_sync(0xffffffffu, myrow, r);
            for (int c = lane; c < R; c += 32) U[row * R + c] = 0.0;
        }
    }
}


// Clears the rows of U_n (and their leverage scores) that the previous update
// left nonzero and the current one (s.touched, counters[2]) does not write.
// A factor that was never updated is cleared entirely, here (dense[n]: must
// precede the writes of the update); otherwise the clearing touches only rows
// that the update does not write, so the step runs it beside the update
// (zero_old_rows, on a side stream once rowbits is set by the hit grouping).
int clear_dense_factor(Session& s, int n, cudaStream_t st) {
    if (!s.dense[n]) return EXAFAC_OK;
    double* sc = s.cfg.sampler == EXAFAC_SAMPLER_CP_ARLS_LEV ? s.scores[n] : nullptr;
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.F.U[n], 0, sizeof(double) * s.dims[n] * s.R, st));
    if (sc) EXAFAC_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(double) * s.dims[n], st));
    return EXAFAC_OK;
}

int zero_old_rows(Session& s, int n, cudaStream_t st) {
    if (s.dense[n]) return EXAFAC_OK;
    double* sc = s.cfg.sampler == EXAFAC_SAMPLER_CP_ARLS_LEV ? s.scores[n] : nullptr;
    zero_rows_kernel<<<152 * 8, 256, 0, st>>>(s.R, s.nzrows[n], s.nzcount + n, s.rowbits, s.F.U[n], sc);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}


// ---------------------------------------------------------------------------
// Exact fit (SparseTensor::compute_exact_fit + compute_2bmb,
// sparse_tensor.hpp:288-356, sort_lookup.hpp:377-438): sum over nonzeros of
// x^2 - 2 x m(x) with m(x) = sum_u sigma_u prod_{k>=1} U_k[i_k,u] * U_0[i_0,u].
// ---------------------------------------------------------------------------
__global__ void fit_kernel(int N, int R, int64_t nnz, const uint32_t* __restrict__ idx, const double* __restrict__ vals,
                           FactorPtrs f, const double* __restrict__ sigma, double* __restrict__ part) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t* c = idx + i * N;
        double value = 0.0;
        for (int u = 0; u < R; u++) {
            double p = sigma[u];
            for (int k = 1; k < N; k++) p *= f.U[k][(int64_t)c[k] * R + u];
            value += p * f.U[0][(int64_t)c[0] * R + u];
        }
        const double x = vals[i];
        acc += x * x - 2 * value * x;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_kernel(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

int fit_residual(Session& s, double* out_dev, cudaStream_t st) {
    const int blocks = 152 * 8;
    fit_kernel<<<blocks, 256, 0, st>>>(s.N, s.R, s.nnz, s.idx, s.vals, factor_ptrs(s), s.F.sigma, s.fitpart); count_launch();
    sum_kernel<<<1, 256, 0, st>>>(s.fitpart, blocks, out_dev); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// U = M * Phi (parallel_dsymm with the full symmetric Phi), warp per row.
__global__ void matmul_rows_kernel(int R, int64_t rows, const double* __restrict__ M, const double* __restrict__ Phi,
                                   double* __restrict__ U) {
    extern __shared__ double sm[];
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* phi = sm;
    double* msm = sm + R * R + w * R;
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) phi[e] = Phi[e];
    __syncthreads();
    for (int64_t r = (int64_t)blockIdx.x * warps + w; r < rows; r += (int64_t)gridDim.x * warps) {
        for (int c = lane; c < R; c += 32) msm[c] = M[r * R + c];
        __syncwarp();
        for (int c = lane; c < R; c += 32) {
            double acc = 0.0;
            for (int k = 0; k < R; k++) acc = fma(msm[k], phi[k * R + c], acc);
            U[r * R + c] = acc;
        }
        __syncwarp();
    }
}

int matmul_rows_sym(Session& s, const double* M, const double* Phi, double* U, int64_t rows, cudaStream_t st) {
    const int R = s.R, warps = 8;
    size_t smem = sizeof(double) * ((size_t)R * R + warps * R);
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(matmul_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    matmul_rows_kernel<<<grid_cap(rows, warps), warps * 32, smem, st>>>(R, rows, M, Phi, U); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// Hadamard product of the per-mode Grams in s.gram, skipping `skip` (-1: none)
// (chain_had_prod, common.h:521-545).
__global__ void chain_kernel(int N, int R, int skip, const double* __restrict__ gram, double* __restrict__ out) {
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        double acc = 1.0;
        for (int k = 0; k < N; k++)
            if (k != skip) acc *= gram[(int64_t)k * R * R + e];
        out[e] = acc;
    }
}

int chain_gram(Session& s, int skip, double* out, cudaStream_t st) {
    chain_kernel<<<1, 256, 0, st>>>(s.N, s.R, skip, s.gram, out); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

}  // namespace exafac
