// STS-CP draws of the mixed forms, breadth first (STS_CP::KRPDrawSamples,
// sts_cp.hpp:203-300, and PartitionTree::PTSample, partition_tree.hpp:
// 204-380, at one rank), in FP32 over the FP32 copies of the trees, factors,
// eigenvector rows and Phi.
//
// A depth-first descent reads one R x R node per level per sample from L2 or
// HBM (P = R (R + 1) / 2 values, 33 KB at R = 128): about 6 TB per sweep of
// the 5-mode, R = 128, J = 2^19 workload.  Here all J samples of a tree move
// one level at a time.  The sample slots are kept ordered by their current
// node (a stable partition after every level, lefts before rights within a
// parent), so a block that takes 64 consecutive slots meets a few runs of
// equal node; it stages each run's node once in shared memory as a full
// symmetric matrix and every warp evaluates x^T A x for its samples of the
// run (y = A x with lanes over columns, 16-byte loads of A's rows).  A level
// then reads each sample's R-vector once and each node once per run.  The
// leaf stage stages the leaf's F x R rows of U (transposed) the same way and
// picks the row by the prefix of its squared dots, in row order.
//
// Per level: the quadratic forms and the branch decisions (one kernel), an
// exclusive scan of the decisions, the children's slot ranges, and the
// scatter of the slots.  The quantities and comparisons are those of the
// depth-first form (cutoff = low + m_L / m); the sums run in a fixed order,
// so the draws repeat run to run.
#include "engine.cuh"
#include "prims.cuh"
#include "umma.cuh"

namespace exafac {

constexpr int kBfsTile = 64;   // slots per block in the level and leaf kernels
constexpr int kBfsWarps = 8;
constexpr int kBfsBlocks = 152 * 3;

__host__ __device__ __forceinline__ int round4(int x) { return (x + 3) & ~3; }

// Run starts of a header of `rows` slots (a multiple of 32) as a bit mask:
// bit i set when slot i begins a run of equal node, or i = n.  One ballot per
// warp of the first rows threads; the caller synchronises before reading.
template <typename T>
__device__ __forceinline__ void run_mask(const T* cs, int n, int rows, uint32_t* mask) {
    const int i = threadIdx.x;
    if (i >= rows) return;
    const bool start = i < n ? (i == 0 || cs[i] != cs[i - 1]) : i == n;
    const uint32_t b = __ballot_sync(0xffffffffu, start);
    if ((i & 31) == 0) mask[i >> 5] = b;
}
// The end of the run that starts at i0: the next run start after i0, or n.
__device__ __forceinline__ int run_end(const uint32_t* mask, int words, int i0, int n) {
    for (int w = (i0 + 1) >> 5; w < words; w++) {
        uint32_t bits = mask[w];
        if (w == ((i0 + 1) >> 5)) bits &= ~0u << ((i0 + 1) & 31);
        if (bits) {
            const int i = (w << 5) + __ffs(bits) - 1;
            return i < n ? i : n;
        }
    }
    return n;
}

// MODE 0: the mass x^T G_0 x of the node G (one node) into mroot[j].
// MODE 1: a level of the descent: the left child's mass m_L, the branch
//         (d <= low + m_L / m goes left), node, (low, high), flag[slot].
// MODE 2: the tail level: as MODE 1 for samples at internal nodes; samples
//         already at a leaf stay (flag 1).
// MODE 3: x^T G_c x with c = node[j] into mroot[j] (the quadratic forms alone,
//         for tests).
// order == nullptr: slot s holds sample s.
template <int MODE>
__global__ void __launch_bounds__(kBfsWarps * 32) bfs_level_kernel(int R, int Pf, const float* __restrict__ G,
                                                                   const float* __restrict__ X, int64_t J,
                                                                   const int32_t* __restrict__ order,
                                                                   int64_t* __restrict__ node,
                                                                   float2* __restrict__ lh, float* __restrict__ mroot,
                                                                   const double* __restrict__ dv,
                                                                   uint32_t* __restrict__ flag, TreeShape t) {
    extern __shared__ __align__(16) float bfs_sm[];
    const int AS = round4(R);
    float* A = bfs_sm;        // R x AS: the run's node, full symmetric
    float* xs = A + R * AS;   // per warp: the sample's vector
    __shared__ int64_t cs[kBfsTile];
    __shared__ int32_t js[kBfsTile];
    __shared__ uint32_t rmask[kBfsTile / 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* xw = xs + w * AS;
    const int b0 = 4 * lane;
    const int64_t ntiles = (J + kBfsTile - 1) / kBfsTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t s0 = tile * kBfsTile;
        const int n = (int)min((int64_t)kBfsTile, J - s0);
        __syncthreads();  // the previous tile is done with cs / js
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int32_t j = order ? order[s0 + i] : (int32_t)(s0 + i);
            js[i] = j;
            cs[i] = MODE == 0 ? 0 : node[j];
        }
        __syncthreads();
        run_mask(cs, n, kBfsTile, rmask);
        __syncthreads();
        for (int i0 = 0; i0 < n;) {  // runs of equal node (uniform over the block)
            const int64_t c = cs[i0];
            const int i1 = run_end(rmask, kBfsTile / 32, i0, n);
            const bool stay = MODE == 2 && tree_is_leaf(t, c);
            if (stay) {
                for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) flag[s0 + i] = 1u;
                i0 = i1;
                continue;
            }
            const int64_t g = MODE == 0 ? 0 : (MODE == 3 ? c : 2 * c + 1);
            const float* Gn = G + g * Pf;
            for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
                const int a = e / R, b = e - a * R;
                A[a * AS + b] = __ldg(Gn + (a <= b ? packed_index(R, a, b) : packed_index(R, b, a)));
            }
            __syncthreads();
            for (int i = i0 + w; i < i1; i += kBfsWarps) {
                const int32_t j = js[i];
                for (int r = lane; r < R; r += 32) xw[r] = X[(int64_t)j * R + r];
                __syncwarp();
                float part = 0.0f;
                if (b0 < R) {
                    float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
                    for (int a = 0; a < R; a++) {
                        const float xa = xw[a];
                        const float4 av = *reinterpret_cast<const float4*>(A + a * AS + b0);
                        y.x = __fmaf_rn(av.x, xa, y.x);
                        y.y = __fmaf_rn(av.y, xa, y.y);
                        y.z = __fmaf_rn(av.z, xa, y.z);
                        y.w = __fmaf_rn(av.w, xa, y.w);
                    }
                    part = y.x * xw[b0];  // columns past R are not added
                    if (b0 + 1 < R) part = __fmaf_rn(y.y, xw[b0 + 1], part);
                    if (b0 + 2 < R) part = __fmaf_rn(y.z, xw[b0 + 2], part);
                    if (b0 + 3 < R) part = __fmaf_rn(y.w, xw[b0 + 3], part);
                }
                const float q = warp_sum(part);
                if (lane == 0) {
                    if (MODE == 0 || MODE == 3) {
                        mroot[j] = q;
                    } else {
                        const float2 bnd = lh[j];
                        const float cutoff = bnd.x + q / mroot[j];
                        const bool left = (float)dv[j] <= cutoff;
                        node[j] = left ? 2 * c + 1 : 2 * c + 2;
                        lh[j] = left ? make_float2(bnd.x, cutoff) : make_float2(cutoff, bnd.y);
                        flag[s0 + i] = left ? 1u : 0u;
                    }
                }
                __syncwarp();
            }
            __syncthreads();  // before the next run restages A
            i0 = i1;
        }
    }
}

// ---------------------------------------------------------------------------
// The level and leaf stages on the fifth-generation tensor cores (R >= 32).
// A block takes 128 consecutive slots (the MMA's M).  For each run of equal
// node in them it forms Y = X B^T (128 x N) with tcgen05.mma, FP32
// accumulators in tensor memory, and reads each sample's row back in the warps
// that own its TMEM lane.  Operands are split into TF32 parts, v = v_hi +
// v_lo (each rounded to TF32), for FP32 accuracy:
// - a level: B = the node's R x R Gram A, symmetric.  Y = X_hi (A_hi + A_lo)
//   ~ A x_hi, and q = sum_c Y[c] (x_hi[c] + 2 x_lo[c]) = x^T A x - x_lo^T A
//   x_lo: two MMAs per K step, no x_lo tile, error ~2^-22 of x^T |A| x plus
//   the FP32 sums (x re-read from L2 for the sum);
// - the leaf stage: B = the leaf's F rows of U, Y[r] = U_r . x ~ X_hi U_hi +
//   X_hi U_lo + X_lo U_hi (three MMAs per K step), then the squared dots and
//   their prefix.
// Operands are staged by the block's threads into the K-major layout of
// umma.cuh: the slots' vectors once per tile (128 x Rk), B in K chunks (Rn x
// KC; 32 for a level, so that a level block's ~100 KB of shared memory lets
// two blocks share an SM, 64 for the leaf stage), a node read from its packed
// FP32 copy.  Rows of a run's MMA that belong to other runs are computed and
// ignored.  Every wait on the MMA barrier is bounded; a wait that runs out
// records EXAFAC_ERR_TIMEOUT, and the block waits once more (bounded) for its
// MMAs, frees its tensor memory and leaves.
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;
constexpr int kTcThreads = 512;

struct TcLayout {
    int Rk, Rn, KC;    // K and N padded to 16, K chunk of B
    bool split_a;      // an x_lo tile (the leaf stage) or not (a level)
    uint32_t a_bytes;  // one slot tile: 128 x Rk
    uint32_t b_bytes;  // one B chunk (hi or lo): Rn x KC
    uint32_t ncols;    // TMEM columns (power of two >= Rn)
};
__host__ __device__ inline TcLayout tc_layout(int R, bool split_a) {
    TcLayout L;
    L.Rn = (R + 15) & ~15;
    L.Rk = L.Rn;
    const int kc = split_a ? 64 : 32;
    L.KC = L.Rk < kc ? L.Rk : kc;
    L.split_a = split_a;
    L.a_bytes = (uint32_t)kTcRows * (uint32_t)L.Rk * 4u;
    L.b_bytes = (uint32_t)L.Rn * (uint32_t)L.KC * 4u;
    L.ncols = L.Rn <= 32 ? 32u : (L.Rn <= 64 ? 64u : (L.Rn <= 128 ? 128u : 256u));
    return L;
}
static size_t tc_smem(int R, bool split_a) {  // + alignment of the base to 1 KB
    const TcLayout L = tc_layout(R, split_a);
    return (split_a ? 2 : 1) * (size_t)L.a_bytes + 2 * (size_t)L.b_bytes + 1024;
}
size_t bfs_leaf_tc_smem(int R) { return tc_smem(R, true); }

// Byte offset of element (r, k) in a K-major tile with 8-row groups sbo bytes apart.
__device__ __forceinline__ uint32_t kmajor_off(int r, int k, uint32_t sbo) {
    return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 2) * 128u + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

// The block's tensor-core state: operand tiles, TMEM accumulator, MMA barrier.
struct TcBlock {
    TcLayout L;
    unsigned char *Ahi, *Alo, *Bhi, *Blo;  // Alo null for a level
    uint32_t sboA, sboB, tmem, idesc, phase, polls;
    uint64_t* bar;
    int* abort_flag;
};

// Allocates TMEM (warp 0), initialises the barrier; every thread returns the same state.
__device__ __forceinline__ TcBlock tc_begin(int R, bool split_a, unsigned char* raw, uint64_t* bar,
                                            uint32_t* tmem_base, int* abort_flag, uint32_t polls) {
    TcBlock b;
    b.L = tc_layout(R, split_a);
    unsigned char* base = raw + ((1024u - (smem_u32(raw) & 1023u)) & 1023u);
    b.Ahi = base;
    b.Alo = split_a ? base + b.L.a_bytes : nullptr;
    b.Bhi = base + (split_a ? 2 : 1) * b.L.a_bytes;
    b.Blo = b.Bhi + b.L.b_bytes;
    b.sboA = (uint32_t)b.L.Rk * 32u;
    b.sboB = (uint32_t)b.L.KC * 32u;
    b.idesc = umma_idesc_tf32(kTcRows, b.L.Rn);
    b.phase = 0;
    b.polls = polls;
    b.bar = bar;
    b.abort_flag = abort_flag;
    if ((threadIdx.x >> 5) == 0) tmem_alloc(tmem_base, b.L.ncols);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        *abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    b.tmem = *tmem_base;
    return b;
}

// Frees TMEM; after an abort, first waits once more (bounded) for the MMAs in
// flight and records the timeout.
__device__ __forceinline__ void tc_end(TcBlock& b, DeviceStatus* status, int where) {
    if (*b.abort_flag) {
        if (threadIdx.x == 0) report(status, EXAFAC_ERR_TIMEOUT, where, blockIdx.x, 0);
        mbar_wait_limited(b.bar, b.phase, b.polls);
    }
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        tc_fence_after();
        tmem_dealloc(b.tmem, b.L.ncols);
    }
}

// Staging loops issue all of a thread's loads of one round (kTcUnroll
// 16-byte chunks) before converting and storing any: the sources are
// gathers from L2 and HBM.  The row index runs fastest across the threads:
// rows of a core matrix are 16 bytes apart, so a warp's 16-byte stores fill 4
// whole 128-byte wavefronts (with the K index fastest, the 32 stores would be
// 128 bytes apart, all in the same banks).
constexpr int kTcUnroll = 8;


// v into hi_tile as FP32 (the tensor core keeps its TF32 part: the value
// truncated to 10 explicit mantissa bits) and, when lo_tile is not null, the
// value minus that truncation (exact in FP32) into lo_tile.
__device__ __forceinline__ float tf32_trunc(float v) { return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u); }
__device__ __forceinline__ void tc_store_split(unsigned char* hi_tile, unsigned char* lo_tile, uint32_t off, float4 v) {
    *reinterpret_cast<float4*>(hi_tile + off) = v;
    if (lo_tile)
        *reinterpret_cast<float4*>(lo_tile + off) =
            make_float4(v.x - tf32_trunc(v.x), v.y - tf32_trunc(v.y), v.z - tf32_trunc(v.z), v.w - tf32_trunc(v.w));
}

// x of a slot, columns k .. k + 3 (zero past R).
__device__ __forceinline__ float4 load_x4(const float* __restrict__ xr, int k, int R, bool vec) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (k < R) {
        if (vec) {
            v = __ldg(reinterpret_cast<const float4*>(xr + k));
        } else {
            v.x = __ldg(xr + k);
            if (k + 1 < R) v.y = __ldg(xr + k + 1);
            if (k + 2 < R) v.z = __ldg(xr + k + 2);
            if (k + 3 < R) v.w = __ldg(xr + k + 3);
        }
    }
    return v;
}

// The tile's slot vectors X[js[r]] (rows past n and columns past R zero).
__device__ __forceinline__ void tc_stage_slots(const TcBlock& b, int R, const float* __restrict__ X,
                                               const int32_t* js, int n) {
    const int total = kTcRows * (b.L.Rk / 4);
    const bool vec = (R & 3) == 0;  // rows start on 16-byte boundaries
    for (int e0 = 0; e0 < total; e0 += kTcThreads * kTcUnroll) {
        float4 v[kTcUnroll];
#pragma unroll
        for (int u = 0; u < kTcUnroll; u++) {
            const int e = e0 + u * kTcThreads + threadIdx.x;
            const int r = e & (kTcRows - 1), k = 4 * (e / kTcRows);
            v[u] = (e < total && r < n) ? load_x4(X + (int64_t)js[r] * R, k, R, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kTcUnroll; u++) {
            const int e = e0 + u * kTcThreads + threadIdx.x;
            if (e < total) tc_store_split(b.Ahi, b.Alo, kmajor_off(e & (kTcRows - 1), 4 * (e / kTcRows), b.sboA), v[u]);
        }
    }
}

// Y (TMEM) = X_hi (B_hi + B_lo)^T (+ X_lo B_hi^T with an x_lo tile) over all
// K chunks, B(nn, k .. k + 3) = load4(nn, k) for nn < Rn, k < Rk a multiple
// of 4 (zero outside the matrix is the loader's job).  Returns false (in
// every thread) when a wait ran out; the caller then ends the block.
template <typename Load4>
__device__ __forceinline__ bool tc_product(TcBlock& b, Load4 load4) {
    const int tid = threadIdx.x;
    for (int k0 = 0; k0 < b.L.Rk; k0 += b.L.KC) {
        const int kc = min(b.L.KC, b.L.Rk - k0);
        const int total = b.L.Rn * (kc / 4);
        for (int e0 = 0; e0 < total; e0 += kTcThreads * kTcUnroll) {
            float4 v[kTcUnroll];
#pragma unroll
            for (int u = 0; u < kTcUnroll; u++) {
                const int e = e0 + u * kTcThreads + tid;
                const int kq = e / b.L.Rn, nn = e - kq * b.L.Rn;
                v[u] = e < total ? load4(nn, k0 + 4 * kq) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < kTcUnroll; u++) {
                const int e = e0 + u * kTcThreads + tid;
                if (e < total) {
                    const int kq = e / b.L.Rn, nn = e - kq * b.L.Rn;
                    tc_store_split(b.Bhi, b.Blo, kmajor_off(nn, 4 * kq, b.sboB), v[u]);
                }
            }
        }
        fence_proxy_async_smem();  // the staged operands, to the tensor core's proxy
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            for (int s = 0; s < kc / 8; s++) {
                const uint32_t aoff = (uint32_t)(k0 + 8 * s) * 32u;  // (k / 4) * 128
                const uint32_t boff = (uint32_t)s * 256u;
                const uint64_t ah = umma_desc(b.Ahi + aoff, 128u, b.sboA);
                const uint64_t bh = umma_desc(b.Bhi + boff, 128u, b.sboB), bl = umma_desc(b.Blo + boff, 128u, b.sboB);
                umma_tf32(b.tmem, ah, bh, b.idesc, (k0 > 0 || s > 0) ? 1u : 0u);
                umma_tf32(b.tmem, ah, bl, b.idesc, 1u);
                if (b.Alo) umma_tf32(b.tmem, umma_desc(b.Alo + aoff, 128u, b.sboA), bh, b.idesc, 1u);
            }
            umma_commit(b.bar);
        }
        // the MMAs have read the chunk (and, after the last, written Y):
        // thread 0 waits on the barrier, the others at the block barrier
        if (tid == 0 && !mbar_wait_limited(b.bar, b.phase, b.polls)) *b.abort_flag = 1;
        __syncthreads();
        if (*b.abort_flag) return false;
        b.phase ^= 1u;
    }
    tc_fence_after();
    return true;
}

// ---- the level kernel: swizzled operands, packed nodes expanded in shared memory

// Level-kernel shapes: N = round16(R) rows of B, K = round32(R) in blocks of
// 32 FP32 values (one 128-byte swizzle row).
struct TcLevelShape {
    int Rn, Rk, nkb, Pf;
    uint32_t a_kb;   // bytes of one K block of the slot tile: 128 rows x 128
    uint32_t b_kb;   // bytes of one K block of one part (hi or lo) of the node: Rn x 128
    uint32_t pk;     // bytes of the packed node buffer (Pf floats, rounded up to 1 KB)
    uint32_t ncols;  // TMEM columns
};
__host__ __device__ inline TcLevelShape tc_level_shape(int R) {
    TcLevelShape L;
    L.Rn = (R + 15) & ~15;
    L.Rk = (R + 31) & ~31;
    L.nkb = L.Rk / 32;
    L.Pf = packed_stride_f32(R);
    L.a_kb = 128u * 128u;
    L.b_kb = (uint32_t)L.Rn * 128u;
    L.pk = ((uint32_t)L.Pf * 4u + 1023u) & ~1023u;
    L.ncols = L.Rn <= 32 ? 32u : (L.Rn <= 64 ? 64u : 128u);
    return L;
}
// Two slot buffers (this tile's, the next tile's in flight), the packed node,
// one node K block (hi and lo parts), 1 KB alignment slack.
size_t bfs_level_tc_smem(int R) {
    const TcLevelShape L = tc_level_shape(R);
    return 2 * (size_t)L.nkb * L.a_kb + L.pk + 2 * (size_t)L.b_kb + 1024;
}

constexpr int kTcLevelThreads = 512;

// The slot vectors X[js[r]] of a tile into a swizzled slot buffer by 16-byte
// asynchronous copies (4-byte ones when rows are not 16-byte aligned), zero
// past R and past the tile's n slots.  The raw FP32 values are the MMA's A
// operand: the tensor core reads an FP32 value as TF32 by dropping its low
// 13 mantissa bits (measured on GB300: the forms from truncated inputs match
// FP64 to ~2.5e-7 of x^T |A| x, from rounded inputs only to ~1.5e-4), so the
// read-back takes x_hi = x with those bits cleared.  One commit group.
__device__ __forceinline__ void tc_issue_slots(unsigned char* A, const float* __restrict__ X, const int32_t* js,
                                               int n, int R, const TcLevelShape& L) {
    const int kqr = L.Rk / 4;
    const bool vec = (R & 3) == 0;
    for (int e = threadIdx.x; e < kTcRows * kqr; e += kTcLevelThreads) {
        const int r = e / kqr, k = 4 * (e - r * kqr);
        unsigned char* dst = A + sw128_off(r, k, L.a_kb);
        const float* row = X + (int64_t)js[r < n ? r : 0] * R;
        if (vec) {
            const bool live = r < n && k < R;
            cp_async16(dst, live ? row + k : X, live ? 16u : 0u);
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const bool live = r < n && k + q < R;
                cp_async4(dst + 4 * q, live ? row + k + q : X, live ? 4u : 0u);
            }
        }
    }
    cp_async_commit();
}

// K block kb of the packed node in shared memory as the B operand: rows n <
// Rn, columns 32 kb .. 32 kb + 31 of the full symmetric matrix, as hi = the
// FP32 value (the tensor core keeps its TF32 part, the value truncated) and
// lo = the value minus its truncation (exact in FP32; the tensor core
// truncates it in turn, ~2^-21 of the entry).  rs[a]: the packed index of
// (a, a).  The row index runs fastest: conflict-free swizzled stores.
__device__ __forceinline__ void tc_expand_kblock(const float* Pk, const int* rs, int R, int kb, unsigned char* Bhi,
                                                 unsigned char* Blo, const TcLevelShape& L) {
    for (int e = threadIdx.x; e < L.Rn * 8; e += kTcLevelThreads) {
        const int c = e / L.Rn, n = e - c * L.Rn;
        const int k0 = kb * 32 + 4 * c;
        float v[4];
        const int rn = n < R ? rs[n] : 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = k0 + q;
            v[q] = (n < R && k < R) ? Pk[k >= n ? rn + (k - n) : rs[k] + (n - k)] : 0.0f;
        }
        const uint32_t off = (uint32_t)n * 128u + (((uint32_t)c ^ ((uint32_t)n & 7u)) * 16u);
        *reinterpret_cast<float4*>(Bhi + off) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4*>(Blo + off) = make_float4(v[0] - tf32_trunc(v[0]), v[1] - tf32_trunc(v[1]),
                                                            v[2] - tf32_trunc(v[2]), v[3] - tf32_trunc(v[3]));
    }
}

template <int MODE>
__global__ void __launch_bounds__(kTcLevelThreads, 1)
    bfs_level_tc_kernel(int R, const float* __restrict__ G, const float* __restrict__ X, int64_t J,
                        const int32_t* __restrict__ order, int64_t* __restrict__ node, float2* __restrict__ lh,
                        float* __restrict__ mroot, const double* __restrict__ dv, uint32_t* __restrict__ flag,
                        TreeShape t, DeviceStatus* status, uint32_t wait_polls) {
    extern __shared__ __align__(16) unsigned char tc_raw[];
    __shared__ int32_t cs2[2][kTcRows];  // current node of each slot (node counts < 2^31)
    __shared__ int32_t js2[2][kTcRows];  // sample of each slot
    __shared__ uint32_t rm2[2][4];       // run starts of each header
    __shared__ float qpart[4][kTcRows];
    __shared__ int rs[kMaxRank];  // packed index of (a, a)
    __shared__ __align__(8) uint64_t bars[2];  // [0] packed node copy, [1] MMAs
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const TcLevelShape L = tc_level_shape(R);
    unsigned char* base = tc_raw + ((1024u - (smem_u32(tc_raw) & 1023u)) & 1023u);
    unsigned char* Abuf[2] = {base, base + L.nkb * L.a_kb};
    float* Pk = reinterpret_cast<float*>(base + 2 * L.nkb * L.a_kb);
    unsigned char* Bhi = base + 2 * L.nkb * L.a_kb + L.pk;
    unsigned char* Blo = Bhi + L.b_kb;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    if (w == 0) tmem_alloc(&tmem_base, L.ncols);
    for (int a = tid; a < R; a += kTcLevelThreads) rs[a] = packed_index(R, a, a);
    if (tid == 0) {
        mbar_init(&bars[0], kTcLevelThreads);  // every thread's node copies
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = umma_idesc_tf32(kTcRows, L.Rn);
    // the packed-node buffer (state kept alike by every thread) and, in
    // thread 0, the MMA barrier's phase
    uint32_t fphase = 0, mphase = 0;
    int64_t pk_node = -1;  // node in (or on its way to) Pk
    bool pk_flight = false;
    // one node into Pk: 16-byte asynchronous copies by every thread, each
    // thread's landing signalled on bars[0] (a single bulk copy of a packed
    // node was measured to land ~8 us after issue, these in time)
    auto issue_node = [&](int64_t g) {
        const float4* src = reinterpret_cast<const float4*>(G + g * L.Pf);
        for (int e = tid; e < L.Pf / 4; e += kTcLevelThreads) cp_async16(Pk + 4 * e, src + e, 16u);
        cp_async_arrive(&bars[0]);
        pk_node = g;
        pk_flight = true;
    };
    // the copy in flight has landed: thread 0 waits on the barrier, the
    // others at the block barrier that follows every call (no spinning warps)
    auto land_node = [&]() -> bool {
        if (!pk_flight) return true;
        pk_flight = false;
        bool ok = true;
        if (tid == 0) ok = mbar_wait_limited(&bars[0], fphase, wait_polls);
        fphase ^= 1u;
        return ok;
    };
    // the node whose Gram a run of current node c multiplies, or -1 for a leaf that stays
    auto run_node = [&](int64_t c) -> int64_t {
        if (MODE == 2 && tree_is_leaf(t, c)) return -1;
        return MODE == 0 ? 0 : (MODE == 3 ? c : 2 * c + 1);
    };
    // the first run needing an MMA among slots [from, n) of a header, or -1
    auto next_run_node = [&](const int32_t* cs, const uint32_t* rm, int from, int n) -> int64_t {
        for (int i = from; i < n; i = run_end(rm, 4, i, n)) {
            const int64_t g = run_node(cs[i]);
            if (g >= 0) return g;
        }
        return -1;
    };
    const int64_t ntiles = (J + kTcRows - 1) / kTcRows;
    const int64_t stride = gridDim.x;
    auto tile_n = [&](int64_t tile) -> int { return (int)min((int64_t)kTcRows, J - tile * kTcRows); };
    // header registers: slot tid of a tile two ahead (threads < 128)
    int32_t hj = 0, hc = 0;
    // prologue: the headers of the first two tiles, the first tile's slot copies
    for (int b = 0; b < 2; b++) {
        const int64_t tile = blockIdx.x + b * stride;
        if (tile < ntiles && tid < tile_n(tile)) {
            const int32_t j = order ? order[tile * kTcRows + tid] : (int32_t)(tile * kTcRows + tid);
            js2[b][tid] = j;
            cs2[b][tid] = MODE == 0 ? 0 : (int32_t)node[j];
        }
    }
    __syncthreads();
    for (int b = 0; b < 2; b++) {
        const int64_t tile = blockIdx.x + b * stride;
        run_mask(cs2[b], tile < ntiles ? tile_n(tile) : 0, kTcRows, rm2[b]);
    }
    __syncthreads();
    if (blockIdx.x < ntiles) tc_issue_slots(Abuf[0], X, js2[0], tile_n(blockIdx.x), R, L);
    int it = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += stride, it++) {
        const int a = it & 1;
        const int64_t s0 = tile * kTcRows;
        const int n = tile_n(tile);
        const int32_t* cs = cs2[a];
        const int32_t* js = js2[a];
        const uint32_t* rm = rm2[a];
        const int64_t t1 = tile + stride, t2 = tile + 2 * stride;
        // the next tile's slot copies (its header is in [a ^ 1]), in flight during this tile
        if (t1 < ntiles) tc_issue_slots(Abuf[a ^ 1], X, js2[a ^ 1], tile_n(t1), R, L);
        else cp_async_commit();  // an empty group keeps the count
        // the header two tiles ahead into registers (its node reads follow below)
        const bool h_live = t2 < ntiles && tid < tile_n(t2);
        if (h_live) hj = order ? order[t2 * kTcRows + tid] : (int32_t)(t2 * kTcRows + tid);
        // this tile's decision inputs (thread i = slot i)
        float2 pl = make_float2(0.f, 0.f);
        float pm = 1.0f;
        double pd = 0.0;
        if ((MODE == 1 || MODE == 2) && tid < n) {
            const int32_t j = js[tid];
            pl = lh[j];
            pm = mroot[j];
            pd = dv[j];
        }
        {  // the first run's node, if not already there (Pk is free only once the copy in flight landed)
            const int64_t g = next_run_node(cs, rm, 0, n);
            if (g >= 0 && g != pk_node) {
                if (pk_flight) {
                    if (!land_node()) abort_flag = 1;
                    __syncthreads();
                }
                issue_node(g);
            }
        }
        cp_async_wait<1>();        // this tile's slot copies (all groups but the newest)
        fence_proxy_async_smem();  // the slot tile, to the tensor core's proxy
        __syncthreads();
        if (abort_flag) goto fail;
        if (h_live) hc = MODE == 0 ? 0 : (int32_t)node[hj];
        unsigned char* A = Abuf[a];
        for (int i0 = 0; i0 < n;) {  // runs of equal node (uniform over the block)
            const int32_t c = cs[i0];
            const int i1 = run_end(rm, 4, i0, n);
            const int64_t g = run_node(c);
            if (g < 0) {
                if (tid >= i0 && tid < i1) flag[s0 + tid] = 1u;
                i0 = i1;
                continue;
            }
            if (pk_node != g) {  // the run's node into Pk (free once the copy in flight landed)
                if (pk_flight) {
                    if (!land_node()) abort_flag = 1;
                    __syncthreads();
                }
                issue_node(g);
            }
            if (!land_node()) abort_flag = 1;
            __syncthreads();
            if (abort_flag) goto fail;
            for (int kb = 0; kb < L.nkb; kb++) {
                tc_expand_kblock(Pk, rs, R, kb, Bhi, Blo, L);
                fence_proxy_async_smem();  // the K block, to the tensor core's proxy
                __syncthreads();
                if (kb + 1 == L.nkb) {  // Pk is free: the next run's node
                    int64_t g2 = next_run_node(cs, rm, i1, n);
                    if (g2 < 0 && t1 < ntiles) g2 = next_run_node(cs2[a ^ 1], rm2[a ^ 1], 0, tile_n(t1));
                    if (g2 >= 0 && g2 != g) issue_node(g2);
                }
                if (tid == 0) {
                    tc_fence_after();
#pragma unroll
                    for (int sub = 0; sub < 4; sub++) {
                        const uint64_t ad = umma_desc_sw128(A + kb * L.a_kb + sub * 32);
                        umma_tf32(tmem, ad, umma_desc_sw128(Bhi + sub * 32), idesc, (kb > 0 || sub > 0) ? 1u : 0u);
                        umma_tf32(tmem, ad, umma_desc_sw128(Blo + sub * 32), idesc, 1u);
                    }
                    umma_commit(&bars[1]);
                    if (!mbar_wait_limited(&bars[1], mphase, wait_polls)) abort_flag = 1;
                    mphase ^= 1u;
                }
                __syncthreads();  // the MMAs are done with the K block (and, after the last, Y is written)
                if (abort_flag) goto fail;
            }
            tc_fence_after();
            {
                // q = sum_c Y[c] (x_hi[c] + 2 x_lo[c]) with x_hi = x truncated
                // to TF32 (what the MMA used); warp w reads lanes 32 (w % 4)
                // .. + 31, column blocks of 16 shared by the four warps of a
                // lane quarter
                const int qw = w & 3, part = w >> 2;
                const int row = qw * 32 + lane;
                float acc = 0.0f;
                for (int cb = part; cb < L.Rn / 16; cb += 4) {
                    float y[16];
                    tmem_ld16(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(cb * 16), y);
#pragma unroll
                    for (int q4 = 0; q4 < 4; q4++) {
                        const float4 x = *reinterpret_cast<const float4*>(A + sw128_off(row, cb * 16 + 4 * q4, L.a_kb));
                        const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                        for (int qq = 0; qq < 4; qq++) {
                            const float h = __uint_as_float(__float_as_uint(xs[qq]) & 0xFFFFE000u);
                            acc = fmaf(y[4 * q4 + qq], fmaf(2.0f, xs[qq] - h, h), acc);
                        }
                    }
                }
                qpart[part][row] = acc;
            }
            tc_fence_before();
            __syncthreads();
            if (tid >= i0 && tid < i1) {  // slot tid, with its prefetched inputs
                const float q = (qpart[0][tid] + qpart[1][tid]) + (qpart[2][tid] + qpart[3][tid]);
                const int32_t j = js[tid];
                if (MODE == 0 || MODE == 3) {
                    mroot[j] = q;
                } else {
                    const float cutoff = pl.x + q / pm;
                    const bool left = (float)pd <= cutoff;
                    node[j] = left ? 2 * (int64_t)c + 1 : 2 * (int64_t)c + 2;
                    lh[j] = left ? make_float2(pl.x, cutoff) : make_float2(cutoff, pl.y);
                    flag[s0 + tid] = left ? 1u : 0u;
                }
            }
            i0 = i1;
        }
        __syncthreads();  // this tile is done with js2 / cs2 [a] and Abuf[a]
        if (h_live) {
            js2[a][tid] = hj;
            cs2[a][tid] = hc;
        }
        __syncthreads();
        run_mask(cs2[a], t2 < ntiles ? tile_n(t2) : 0, kTcRows, rm2[a]);  // read after the next iteration's barriers
    }
    cp_async_wait<0>();
    if (!land_node()) abort_flag = 1;  // a prefetched node no run used
    __syncthreads();
    if (abort_flag) goto fail;
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, L.ncols);
    }
    return;
fail:
    cp_async_wait<0>();  // this thread's copies (the node's included) have landed
    if (tid == 0) {
        report(status, EXAFAC_ERR_TIMEOUT, 20, blockIdx.x, 0);
        // the MMAs in flight may still complete: wait once more (bounded)
        mbar_wait_limited(&bars[1], mphase, wait_polls);
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, L.ncols);
    }
}

// ---- the resident-node level kernel: levels whose nodes each fill many tiles
//
// At the root and the shallow levels a node's slots fill many consecutive
// tiles.  This kernel keeps the node's whole B operand (every K block, hi and
// lo parts: 128 KB at R = 128) in shared memory and expands it again only when
// the node changes; each block takes a contiguous range of tiles so that its
// consecutive tiles share the node.  With B resident the slot tile is single
// buffered: each thread keeps the x values its epilogue needs in registers,
// so the next tile's slot copies start as soon as the MMAs of this tile are
// done and land during the epilogue.  The arithmetic (operands, MMA order,
// epilogue order) is that of bfs_level_tc_kernel: the results are the same
// bit for bit.

// Shared memory: B (every K block, hi and lo parts), one slot tile, 1 KB
// alignment slack.
size_t bfs_level_tcr_smem(int R) {
    const TcLevelShape L = tc_level_shape(R);
    return 2 * (size_t)L.nkb * L.b_kb + (size_t)L.nkb * L.a_kb + 1024;
}

// Average slots per node from which a descent level runs on the
// resident-node kernel (64 tiles).  Below it the slots of a node are skewed
// over fewer tiles, node changes become frequent, and the double-buffered
// slot tiles of bfs_level_tc_kernel win (measured on GB300 at R = 128,
// J = 2^19: the resident kernel 223 us against 266 us at 8192 slots per
// node, 285 against 273 at 4096, 381 against 287 at 1024).
constexpr int64_t kTcrMinSlotsPerNode = 64 * kTcRows;

constexpr int kTcrExpand = (kMaxRank * kMaxRank / 4) / kTcLevelThreads;  // column groups per thread at most

// The whole packed FP32 node P (global memory) as the B operand: hi = the
// value, lo = the value minus its truncation to TF32, every K block.  All of
// a thread's loads are issued before its swizzled stores.
__device__ __forceinline__ void tcr_expand_node(const float* __restrict__ P, const int* rs, int R, unsigned char* Bhi,
                                                unsigned char* Blo, const TcLevelShape& L) {
    const int groups = L.Rn * (L.Rk / 4);  // (row, group of 4 columns), row fastest
    float v[kTcrExpand][4];
#pragma unroll
    for (int it = 0; it < kTcrExpand; it++) {
        const int e = threadIdx.x + it * kTcLevelThreads;
        const int cg = e / L.Rn, n = e - cg * L.Rn;
        const bool row_live = e < groups && n < R;
        const int rn = row_live ? rs[n] : 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = 4 * cg + q;
            v[it][q] = (row_live && k < R) ? __ldg(P + (k >= n ? rn + (k - n) : rs[k] + (n - k))) : 0.0f;
        }
    }
#pragma unroll
    for (int it = 0; it < kTcrExpand; it++) {
        const int e = threadIdx.x + it * kTcLevelThreads;
        if (e < groups) {
            const int cg = e / L.Rn, n = e - cg * L.Rn;
            const uint32_t off = (uint32_t)(cg >> 3) * L.b_kb + (uint32_t)n * 128u +
                                 ((((uint32_t)cg & 7u) ^ ((uint32_t)n & 7u)) * 16u);
            *reinterpret_cast<float4*>(Bhi + off) = make_float4(v[it][0], v[it][1], v[it][2], v[it][3]);
            *reinterpret_cast<float4*>(Blo + off) =
                make_float4(v[it][0] - tf32_trunc(v[it][0]), v[it][1] - tf32_trunc(v[it][1]),
                            v[it][2] - tf32_trunc(v[it][2]), v[it][3] - tf32_trunc(v[it][3]));
        }
    }
}

// MODE 0, 1 and 3 as bfs_level_kernel (MODE 2, whose leaves need no MMA,
// stays on bfs_level_tc_kernel).
template <int MODE>
__global__ void __launch_bounds__(kTcLevelThreads, 1)
    bfs_level_tcr_kernel(int R, const float* __restrict__ G, const float* __restrict__ X, int64_t J,
                         const int32_t* __restrict__ order, int64_t* __restrict__ node, float2* __restrict__ lh,
                         float* __restrict__ mroot, const double* __restrict__ dv, uint32_t* __restrict__ flag,
                         DeviceStatus* status, uint32_t wait_polls) {
    static_assert(MODE == 0 || MODE == 1 || MODE == 3, "the resident-node kernel takes MODE 0, 1 or 3");
    extern __shared__ __align__(16) unsigned char tc_raw[];
    __shared__ int32_t cs2[2][kTcRows];  // current node of each slot
    __shared__ int32_t js2[2][kTcRows];  // sample of each slot
    __shared__ uint32_t rm2[2][4];       // run starts of each header
    __shared__ float qpart[4][kTcRows];
    __shared__ int rs[kMaxRank];  // packed index of (a, a)
    __shared__ __align__(8) uint64_t mbar;  // the MMAs
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const TcLevelShape L = tc_level_shape(R);
    unsigned char* base = tc_raw + ((1024u - (smem_u32(tc_raw) & 1023u)) & 1023u);
    unsigned char* Bhi = base;
    unsigned char* Blo = base + L.nkb * L.b_kb;
    unsigned char* A = base + 2 * L.nkb * L.b_kb;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    if (w == 0) tmem_alloc(&tmem_base, L.ncols);
    for (int a = tid; a < R; a += kTcLevelThreads) rs[a] = packed_index(R, a, a);
    if (tid == 0) {
        mbar_init(&mbar, 1);
        fence_mbar_init();
        abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = umma_idesc_tf32(kTcRows, L.Rn);
    uint32_t mphase = 0;  // thread 0's
    int64_t resident = -1;  // the node B holds (alike in every thread)
    auto run_node = [&](int64_t c) -> int64_t { return MODE == 0 ? 0 : (MODE == 3 ? c : 2 * c + 1); };
    // this block's contiguous range of tiles
    const int64_t ntiles_all = (J + kTcRows - 1) / kTcRows;
    const int64_t per = (ntiles_all + gridDim.x - 1) / gridDim.x;
    const int64_t tfirst = (int64_t)blockIdx.x * per;
    const int64_t tend = min(ntiles_all, tfirst + per);
    auto tile_n = [&](int64_t tile) -> int { return (int)min((int64_t)kTcRows, J - tile * kTcRows); };
    // the epilogue's share: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its
    // rows), column blocks of 16 part, part + 4 (at most two: Rn <= 128)
    const int qw = w & 3, part = w >> 2, row = qw * 32 + lane;
    const int ncb = L.Rn / 16;
    int32_t hj = 0, hc = 0;  // header registers: slot tid of the tile two ahead
    int it = 0;
    for (int b = 0; b < 2; b++) {
        const int64_t tile = tfirst + b;
        if (tile < tend && tid < tile_n(tile)) {
            const int32_t j = order ? order[tile * kTcRows + tid] : (int32_t)(tile * kTcRows + tid);
            js2[b][tid] = j;
            cs2[b][tid] = MODE == 0 ? 0 : (int32_t)node[j];
        }
    }
    __syncthreads();
    for (int b = 0; b < 2; b++) {
        const int64_t tile = tfirst + b;
        run_mask(cs2[b], tile < tend ? tile_n(tile) : 0, kTcRows, rm2[b]);
    }
    __syncthreads();
    if (tfirst < tend) tc_issue_slots(A, X, js2[0], tile_n(tfirst), R, L);
    for (int64_t tile = tfirst; tile < tend; tile++, it++) {
        const int a = it & 1;
        const int64_t s0 = tile * kTcRows;
        const int n = tile_n(tile);
        const int32_t* cs = cs2[a];
        const int32_t* js = js2[a];
        const uint32_t* rm = rm2[a];
        const int64_t t1 = tile + 1, t2 = tile + 2;
        const bool h_live = t2 < tend && tid < tile_n(t2);
        if (h_live) hj = order ? order[t2 * kTcRows + tid] : (int32_t)(t2 * kTcRows + tid);
        float2 pl = make_float2(0.f, 0.f);
        float pm = 1.0f;
        double pd = 0.0;
        if (MODE == 1 && tid < n) {
            const int32_t j = js[tid];
            pl = lh[j];
            pm = mroot[j];
            pd = dv[j];
        }
        cp_async_wait<0>();        // this tile's slot copies
        fence_proxy_async_smem();  // the slot tile, to the tensor core's proxy
        __syncthreads();
        if (h_live) hc = MODE == 0 ? 0 : (int32_t)node[hj];
        // the epilogue's x values as x_hi + 2 x_lo, x_hi = x truncated to
        // TF32 (what the MMA reads)
        float xe[2][16];
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int cb = part + 4 * i;
#pragma unroll
            for (int q4 = 0; q4 < 4; q4++) {
                float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                if (cb < ncb) x = *reinterpret_cast<const float4*>(A + sw128_off(row, cb * 16 + 4 * q4, L.a_kb));
                const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int qq = 0; qq < 4; qq++) {
                    const float h = tf32_trunc(xs[qq]);
                    xe[i][4 * q4 + qq] = fmaf(2.0f, xs[qq] - h, h);
                }
            }
        }
        for (int i0 = 0; i0 < n;) {  // runs of equal node (uniform over the block)
            const int32_t c = cs[i0];
            const int i1 = run_end(rm, 4, i0, n);
            const int64_t g = run_node(c);
            if (g != resident) {  // the MMAs that read B are done
                tcr_expand_node(G + g * L.Pf, rs, R, Bhi, Blo, L);
                fence_proxy_async_smem();
                __syncthreads();
                resident = g;
            }
            if (tid == 0) {
                tc_fence_after();
                for (int kb = 0; kb < L.nkb; kb++) {
#pragma unroll
                    for (int sub = 0; sub < 4; sub++) {
                        const uint64_t ad = umma_desc_sw128(A + kb * L.a_kb + sub * 32);
                        umma_tf32(tmem, ad, umma_desc_sw128(Bhi + kb * L.b_kb + sub * 32), idesc,
                                  (kb > 0 || sub > 0) ? 1u : 0u);
                        umma_tf32(tmem, ad, umma_desc_sw128(Blo + kb * L.b_kb + sub * 32), idesc, 1u);
                    }
                }
                umma_commit(&mbar);
                if (!mbar_wait_limited(&mbar, mphase, wait_polls)) abort_flag = 1;
                mphase ^= 1u;
            }
            __syncthreads();  // the MMAs are done: Y is in TMEM, A and B are free
            if (abort_flag) goto fail;
            tc_fence_after();
            // after the tile's last run the slot buffer takes the next tile
            // (x is in registers); its copies land during this epilogue
            if (i1 >= n && t1 < tend) tc_issue_slots(A, X, js2[a ^ 1], tile_n(t1), R, L);
            {
                float acc = 0.0f;
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const int cb = part + 4 * i;
                    if (cb < ncb) {
                        float y[16];
                        tmem_ld16(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(cb * 16), y);
#pragma unroll
                        for (int q = 0; q < 16; q++) acc = fmaf(y[q], xe[i][q], acc);
                    }
                }
                qpart[part][row] = acc;
            }
            tc_fence_before();
            __syncthreads();
            if (tid >= i0 && tid < i1) {  // slot tid, with its prefetched inputs
                const float q = (qpart[0][tid] + qpart[1][tid]) + (qpart[2][tid] + qpart[3][tid]);
                const int32_t j = js[tid];
                if (MODE == 0 || MODE == 3) {
                    mroot[j] = q;
                } else {
                    const float cutoff = pl.x + q / pm;
                    const bool left = (float)pd <= cutoff;
                    node[j] = left ? 2 * (int64_t)c + 1 : 2 * (int64_t)c + 2;
                    lh[j] = left ? make_float2(pl.x, cutoff) : make_float2(cutoff, pl.y);
                    flag[s0 + tid] = left ? 1u : 0u;
                }
            }
            i0 = i1;
        }
        __syncthreads();  // this tile is done with js2 / cs2 [a] and qpart
        if (h_live) {
            js2[a][tid] = hj;
            cs2[a][tid] = hc;
        }
        __syncthreads();
        run_mask(cs2[a], t2 < tend ? tile_n(t2) : 0, kTcRows, rm2[a]);  // read after the next iteration's barriers
    }
    cp_async_wait<0>();
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, L.ncols);
    }
    return;
fail:
    cp_async_wait<0>();
    if (tid == 0) {
        report(status, EXAFAC_ERR_TIMEOUT, 21, blockIdx.x, 0);
        mbar_wait_limited(&mbar, mphase, wait_polls);  // the MMAs in flight may still complete (bounded)
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, L.ncols);
    }
}

// Leaf stage on the tensor cores (F > 1, F <= Rn): Y[r] = U_r . x for the
// leaf's rows, then for each sample the squared dots' inclusive prefix in row
// order and the first row r < F - 1 with frac x total < prefix_r, else the
// last row the leaf holds (the rule of bfs_leaf_kernel).  All sixteen warps
// share the epilogue: each thread holds one slot's squares for a slice of 32
// leaf rows (two TMEM loads), the slices' sums meet in shared memory, and the
// slice that holds the crossing names the row.
__global__ void __launch_bounds__(kTcThreads, 1)
    bfs_leaf_tc_kernel(int R, TreeShape t, const float* __restrict__ U, const float* __restrict__ X, int64_t J,
                       const int32_t* __restrict__ order, const int64_t* __restrict__ node,
                       const float2* __restrict__ lh, const double* __restrict__ dv, int N, int col,
                       uint32_t* __restrict__ samples, int32_t* __restrict__ empty, DeviceStatus* status,
                       uint32_t wait_polls) {
    extern __shared__ __align__(16) unsigned char tc_raw[];
    __shared__ int64_t cs[kTcRows];
    __shared__ int32_t js[kTcRows];
    __shared__ uint32_t rmask[kTcRows / 32];
    __shared__ float psum[4][kTcRows];  // squared dots summed over each slice of 32 leaf rows
    __shared__ int pick[kTcRows];       // the row each slot takes
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    TcBlock b = tc_begin(R, true, tc_raw, &bar, &tmem_base, &abort_flag, wait_polls);
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int F = (int)t.F;
    const int64_t ntiles = (J + kTcRows - 1) / kTcRows;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t s0 = tile * kTcRows;
        const int n = (int)min((int64_t)kTcRows, J - s0);
        __syncthreads();
        for (int i = tid; i < n; i += kTcThreads) {
            const int32_t j = order[s0 + i];
            js[i] = j;
            cs[i] = node[j];
        }
        __syncthreads();
        tc_stage_slots(b, R, X, js, n);
        run_mask(cs, n, kTcRows, rmask);
        __syncthreads();
        for (int i0 = 0; i0 < n;) {
            const int64_t c = cs[i0];
            const int i1 = run_end(rmask, kTcRows / 32, i0, n);
            const int64_t leaf = tree_leaf_idx(t, c);
            const int rows = (int)min((int64_t)F, t.n - leaf * F);
            const float* Ub = U + leaf * F * R;
            const bool vec = (R & 3) == 0;
            const bool ok = tc_product(b, [&](int r, int k) -> float4 {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r < rows && k < R) {
                    const float* u = Ub + (int64_t)r * R + k;
                    if (vec) {
                        v = __ldg(reinterpret_cast<const float4*>(u));
                    } else {
                        v.x = __ldg(u);
                        if (k + 1 < R) v.y = __ldg(u + 1);
                        if (k + 2 < R) v.z = __ldg(u + 2);
                        if (k + 3 < R) v.w = __ldg(u + 3);
                    }
                }
                return v;
            });
            if (!ok) {
                tc_end(b, status, 21);
                return;
            }
            {
                // Every warp: lane quarter qw (slots 32 qw .. + 31) and a
                // slice of 32 leaf rows (columns of Y).  The squared dots'
                // slice sums go through shared memory; the slot's total and
                // the sums before each slice follow, and the one slice whose
                // range [before, before + sum) holds frac x total reports the
                // first row r < F - 1 of it with frac x total < prefix_r
                // (the inverse-CDF pick of the row in row order).
                const int qw = w & 3, part = w >> 2;
                const int row = qw * 32 + lane;  // this thread's slot in the tile
                const int c0 = part * 32;
                const int nb = b.L.Rn / 16;
                const int fr = min(F, b.L.Rn);   // leaf rows that have a column
                const uint32_t tl = b.tmem + ((uint32_t)(qw * 32) << 16);
                float y[2][16];
                float ps = 0.0f;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int cb = 2 * part + h;
                    if (cb < nb) {
                        tmem_ld16(tl + (uint32_t)(cb * 16), y[h]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 16; q++) y[h][q] = 0.0f;
                    }
#pragma unroll
                    for (int q = 0; q < 16; q++)
                        if (c0 + 16 * h + q < fr) ps = fmaf(y[h][q], y[h][q], ps);
                }
                psum[part][row] = ps;
                if (part == 0) pick[row] = F - 1;
                __syncthreads();
                const bool mine = row >= i0 && row < i1;
                const int32_t j = mine ? js[row] : 0;
                float before = 0.0f, total = 0.0f;
#pragma unroll
                for (int p = 0; p < 4; p++) {
                    if (p == part) before = total;
                    total += psum[p][row];
                }
                const bool is_empty = !(total > 0.0f);
                if (mine && !is_empty && c0 < fr) {
                    const float2 bnd = lh[j];
                    const float frac = ((float)dv[j] - bnd.x) / (bnd.y - bnd.x);
                    const float thr = frac * total;
                    const bool last_slice = c0 + 32 >= fr;
                    const bool lo_ok = part == 0 || thr >= before;
                    const bool hi_ok = last_slice || thr < before + psum[part][row];
                    if (lo_ok && hi_ok) {
                        int res = min(c0 + 31, fr - 1);  // rounding: the slice's last row
                        if (last_slice) res = F - 1;
                        float prefix = before;
                        bool found = false;
#pragma unroll
                        for (int h = 0; h < 2; h++) {
#pragma unroll
                            for (int q = 0; q < 16; q++) {
                                const int r = c0 + 16 * h + q;
                                prefix = fmaf(y[h][q], y[h][q], prefix);
                                if (!found && r < F - 1 && r < fr && thr < prefix) {
                                    res = r;
                                    found = true;
                                }
                            }
                        }
                        pick[row] = res;
                    }
                }
                __syncthreads();
                if (mine && part == 0) {
                    const int rows_here = rows;
                    int res = pick[row];
                    if (is_empty) res = 0;
                    else if (res >= rows_here) res = rows_here - 1;  // frac >= 1 in a partial leaf
                    samples[(int64_t)j * N + col] = (uint32_t)(leaf * F + res);
                    if (is_empty) empty[j] = 1;
                }
            }
            tc_fence_before();
            __syncthreads();
            i0 = i1;
        }
    }
    tc_end(b, status, 21);
}

// Slot ranges of the next level's nodes from the parents' (nl of them,
// ranges off[0..nl]) and the exclusive scan SL of the flags (SL[J] = total):
// the left child takes the parent's first nleft slots.
__global__ void bfs_offsets_kernel(int64_t nl, int64_t J, const int64_t* __restrict__ off,
                                   const int64_t* __restrict__ SL, int64_t* __restrict__ coff) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t start = off[i], end = off[i + 1];
        coff[2 * i] = start;
        coff[2 * i + 1] = start + (SL[end] - SL[start]);
        if (i == 0) coff[2 * nl] = J;
    }
}

// The stable partition: within its parent's range, a slot whose flag is set
// (went left, or stayed at a leaf on the tail level) keeps its order among
// those, before the others.  lb: the parents' first node index.
__global__ void bfs_scatter_kernel(int64_t J, int64_t lb, int64_t nl, const int32_t* __restrict__ order,
                                   const int64_t* __restrict__ node, const int64_t* __restrict__ off,
                                   const int64_t* __restrict__ SL, const uint32_t* __restrict__ flag,
                                   int32_t* __restrict__ order2) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < J; s += (int64_t)gridDim.x * blockDim.x) {
        const int32_t j = order[s];
        const int64_t c = node[j];
        const int64_t parent = c >= lb + nl ? (c - 1) / 2 : c;
        const int64_t i = parent - lb;
        const int64_t start = off[i], end = off[i + 1];
        const int64_t before = SL[s] - SL[start];
        const int64_t nleft = SL[end] - SL[start];
        const int64_t pos = flag[s] ? start + before : start + nleft + ((s - start) - before);
        order2[pos] = j;
    }
}

// Every sample at the root: node 0, (low, high) = (0, 1); the root's range
// is all slots.
__global__ void bfs_reset_kernel(int64_t J, int64_t* __restrict__ node, float2* __restrict__ lh,
                                 int32_t* __restrict__ order, int64_t* __restrict__ off, int first) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < J; s += (int64_t)gridDim.x * blockDim.x) {
        node[s] = 0;
        lh[s] = make_float2(0.0f, 1.0f);
        if (first) order[s] = (int32_t)s;
        if (s == 0) {
            off[0] = 0;
            off[1] = J;
        }
    }
}

// Leaf stage, F > 1: runs of equal leaf; the leaf's rows of U staged
// transposed (UT[a][r], rows past the tensor zero); per sample the squared
// dots q_r^2 = (U_r . x)^2 (lanes over rows, four each), their inclusive
// prefix in row order, and the first row r < F - 1 with frac < prefix_r /
// total, else the last row the leaf holds.  A leaf of zero total marks the
// sample empty (weight 0) and takes its first row.
__global__ void __launch_bounds__(kBfsWarps * 32) bfs_leaf_kernel(int R, TreeShape t, const float* __restrict__ U,
                                                                  const float* __restrict__ X, int64_t J,
                                                                  const int32_t* __restrict__ order,
                                                                  const int64_t* __restrict__ node,
                                                                  const float2* __restrict__ lh,
                                                                  const double* __restrict__ dv, int N, int col,
                                                                  uint32_t* __restrict__ samples,
                                                                  int32_t* __restrict__ empty) {
    extern __shared__ __align__(16) float bfs_sm[];
    const int F = (int)t.F;
    const int FS = round4(F) + 4;  // UT row stride
    const int AS = round4(R);
    float* UT = bfs_sm;          // R x FS
    float* xs = UT + R * FS;     // per warp
    __shared__ int64_t cs[kBfsTile];
    __shared__ int32_t js[kBfsTile];
    __shared__ uint32_t rmask[kBfsTile / 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* xw = xs + w * AS;
    const int r0 = 4 * lane;
    const int64_t ntiles = (J + kBfsTile - 1) / kBfsTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t s0 = tile * kBfsTile;
        const int n = (int)min((int64_t)kBfsTile, J - s0);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int32_t j = order[s0 + i];
            js[i] = j;
            cs[i] = node[j];
        }
        __syncthreads();
        run_mask(cs, n, kBfsTile, rmask);
        __syncthreads();
        for (int i0 = 0; i0 < n;) {
            const int64_t c = cs[i0];
            const int i1 = run_end(rmask, kBfsTile / 32, i0, n);
            const int64_t leaf = tree_leaf_idx(t, c);
            const int rows = (int)min((int64_t)F, t.n - leaf * F);
            const float* Ub = U + leaf * F * R;
            for (int e = threadIdx.x; e < F * R; e += blockDim.x) {
                const int r = e / R, a = e - r * R;
                UT[a * FS + r] = r < rows ? __ldg(Ub + (int64_t)r * R + a) : 0.0f;
            }
            __syncthreads();
            for (int i = i0 + w; i < i1; i += kBfsWarps) {
                const int32_t j = js[i];
                for (int r = lane; r < R; r += 32) xw[r] = X[(int64_t)j * R + r];
                __syncwarp();
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r0 < F) {
#pragma unroll 4
                    for (int a = 0; a < R; a++) {
                        const float xa = xw[a];
                        const float4 uv = *reinterpret_cast<const float4*>(UT + a * FS + r0);
                        q.x = __fmaf_rn(uv.x, xa, q.x);
                        q.y = __fmaf_rn(uv.y, xa, q.y);
                        q.z = __fmaf_rn(uv.z, xa, q.z);
                        q.w = __fmaf_rn(uv.w, xa, q.w);
                    }
                }
                // squared dots of this lane's rows (rows past F add nothing)
                float p0 = r0 < F ? q.x * q.x : 0.0f;
                float p1 = r0 + 1 < F ? q.y * q.y : 0.0f;
                float p2 = r0 + 2 < F ? q.z * q.z : 0.0f;
                float p3 = r0 + 3 < F ? q.w * q.w : 0.0f;
                p1 += p0;
                p2 += p1;
                p3 += p2;
                float inc = p3;  // inclusive scan of the lanes' totals
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const float u = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += u;
                }
                const float before = inc - p3;
                const float total = __shfl_sync(0xffffffffu, inc, 31);
                int res;
                bool is_empty = false;
                if (!(total > 0.0f)) {
                    is_empty = true;
                    res = 0;
                } else {
                    const float2 bnd = lh[j];
                    const float frac = ((float)dv[j] - bnd.x) / (bnd.y - bnd.x);
                    int mine = 128;  // this lane's first hit among its rows r < F - 1
                    if (r0 < F - 1 && frac < (before + p0) / total) mine = r0;
                    else if (r0 + 1 < F - 1 && frac < (before + p1) / total) mine = r0 + 1;
                    else if (r0 + 2 < F - 1 && frac < (before + p2) / total) mine = r0 + 2;
                    else if (r0 + 3 < F - 1 && frac < (before + p3) / total) mine = r0 + 3;
                    const unsigned mask = __ballot_sync(0xffffffffu, mine < 128);
                    res = mask ? __shfl_sync(0xffffffffu, mine, __ffs(mask) - 1) : F - 1;
                    if (res >= rows) res = rows - 1;  // frac >= 1 in a partial leaf
                }
                if (lane == 0) {
                    samples[(int64_t)j * N + col] = (uint32_t)(leaf * F + res);
                    if (is_empty) empty[j] = 1;
                }
                __syncwarp();
            }
            __syncthreads();
            i0 = i1;
        }
    }
}

// Leaf stage, F = 1 (eigen trees): the leaf index.
__global__ void bfs_leaf1_kernel(TreeShape t, int64_t J, const int64_t* __restrict__ node, int N, int col,
                                 uint32_t* __restrict__ samples, int32_t* __restrict__ v_out) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < J; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = tree_leaf_idx(t, node[j]);
        samples[j * N + col] = (uint32_t)v;
        v_out[j] = (int32_t)v;
    }
}

// sh = h * E_next[v] and h = h * U_k[row] (row-wise products), h = 1.
// sh[j] = h[j] * E[v[j]] and h[j] *= U[row of j], elementwise over R: a warp
// per sample row, 16-byte accesses along the row when the rows are 16-byte
// aligned (one multiply per element either way, as before).
__device__ __forceinline__ void row_product(int R, const float* a, const float* __restrict__ b, float* out) {
    const int lane = threadIdx.x & 31;
    if ((R & 3) == 0 && (((uintptr_t)a | (uintptr_t)b | (uintptr_t)out) & 15u) == 0) {
        for (int c = 4 * lane; c < R; c += 128) {
            const float4 x = *reinterpret_cast<const float4*>(a + c);
            const float4 y = __ldg(reinterpret_cast<const float4*>(b + c));
            *reinterpret_cast<float4*>(out + c) = make_float4(x.x * y.x, x.y * y.y, x.z * y.z, x.w * y.w);
        }
    } else {
        for (int c = lane; c < R; c += 32) out[c] = a[c] * __ldg(b + c);
    }
}

__global__ void bfs_scale_kernel(int R, int64_t J, const float* __restrict__ h, const float* __restrict__ Ek,
                                 const int32_t* __restrict__ v, float* __restrict__ sh) {
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < J; j += nw)
        row_product(R, h + j * R, Ek + (int64_t)v[j] * R, sh + j * R);
}

__global__ void bfs_row_update_kernel(int R, int64_t J, const float* __restrict__ Uk, const uint32_t* __restrict__ samples,
                                      int N, int col, float* __restrict__ h) {
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < J; j += nw)
        row_product(R, h + j * R, Uk + (int64_t)samples[j * N + col] * R, h + j * R);
}

__global__ void bfs_init_kernel(int R, int64_t J, float* __restrict__ h, int32_t* __restrict__ empty) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < J * R; e += (int64_t)gridDim.x * blockDim.x) {
        h[e] = 1.0f;
        if (e < J) empty[e] = 0;
    }
}

// Weight = R / (J h^T Phi h); zero for a sample whose descent ended in an
// empty leaf or whose quadratic form rounded to zero or below.
__global__ void bfs_weight_kernel(int R, int64_t J, const float* __restrict__ hq, const int32_t* __restrict__ empty,
                                  double* __restrict__ weights) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < J; j += (int64_t)gridDim.x * blockDim.x) {
        const float q = hq[j];
        weights[j] = (!empty[j] && q > 0.0f) ? (double)R / ((double)q * (double)J) : 0.0;
    }
}

static unsigned grid_for_elems(int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 152 * 16));
}

size_t bfs_level_smem(int R) { return sizeof(float) * ((size_t)R * round4(R) + (size_t)kBfsWarps * round4(R)); }
size_t bfs_leaf_smem(int R, int F) {
    return sizeof(float) * ((size_t)R * (round4(F) + 4) + (size_t)kBfsWarps * round4(R));
}

static void bfs_set_smem_limits() {
    static bool done = false;  // host-side, per process: the attributes hold for every device's context
    if (done) return;
    const int lsm = (int)bfs_level_smem(kMaxRank), fsm = (int)bfs_leaf_smem(kMaxRank, kMaxRank);
    const int tsm = (int)bfs_level_tc_smem(kMaxRank), tlsm = (int)bfs_leaf_tc_smem(kMaxRank);
    cudaFuncSetAttribute(bfs_level_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, lsm);
    cudaFuncSetAttribute(bfs_level_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, lsm);
    cudaFuncSetAttribute(bfs_level_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lsm);
    cudaFuncSetAttribute(bfs_level_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, lsm);
    cudaFuncSetAttribute(bfs_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm);
    cudaFuncSetAttribute(bfs_level_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
    cudaFuncSetAttribute(bfs_level_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
    cudaFuncSetAttribute(bfs_level_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
    cudaFuncSetAttribute(bfs_level_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
    cudaFuncSetAttribute(bfs_leaf_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tlsm);
    const int rsm = (int)bfs_level_tcr_smem(kMaxRank);
    cudaFuncSetAttribute(bfs_level_tcr_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm);
    cudaFuncSetAttribute(bfs_level_tcr_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm);
    cudaFuncSetAttribute(bfs_level_tcr_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm);
    done = true;
}

// One level (MODE as bfs_level_kernel) over slots order[0 .. J) of the packed
// FP32 nodes G: on the tensor cores when use_tc (R >= kTcMinRank), with the
// node kept resident when `resident` (long runs: the root and shallow levels;
// MODE 0, 1 and 3), else on the CUDA cores.
template <int MODE>
static void bfs_level_launch(bool use_tc, bool resident, int R, const float* G, const float* X, int64_t J,
                             const int32_t* order, int64_t* node, float2* lh, float* m, const double* dv,
                             uint32_t* flag, const TreeShape& t, DeviceStatus* status, uint32_t polls,
                             cudaStream_t st) {
    const int Pf = packed_stride_f32(R);
    if (use_tc && resident && MODE != 2) {
        const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(J, kTcRows), 152));
        bfs_level_tcr_kernel<MODE == 2 ? 1 : MODE><<<blocks, kTcLevelThreads, bfs_level_tcr_smem(R), st>>>(
            R, G, X, J, order, node, lh, m, dv, flag, status, polls);
    } else if (use_tc) {
        const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(J, kTcRows), 152));
        bfs_level_tc_kernel<MODE><<<blocks, kTcLevelThreads, bfs_level_tc_smem(R), st>>>(R, G, X, J, order, node, lh,
                                                                                       m, dv, flag, t, status, polls);
    } else {
        const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(J, kBfsTile), kBfsBlocks));
        bfs_level_kernel<MODE><<<blocks, kBfsWarps * 32, bfs_level_smem(R), st>>>(R, Pf, G, X, J, order, node, lh, m,
                                                                                 dv, flag, t);
    }
    count_launch();
}

// One descent of every sample through tree t (node array G, stride Pf;
// leaf rows U for F > 1), driven by x (J x R) and the uniforms dv[j]; the
// chosen rows go to samples[j * N + col] (and v_out for F = 1).
static int bfs_descend(Session& s, const TreeShape& t, const float* G, const float* U, const float* X,
                       const double* dv, int64_t J, int col, int32_t* v_out, cudaStream_t st) {
    const int R = s.R, Pf = packed_stride_f32(R);
    BfsState& b = s.bfs;
    const bool tc = R >= kTcMinRank;
    const uint32_t polls = s.wait_polls ? s.wait_polls : kSpinLimit;
    // every descent starts from the identity order (a permutation of 0..J-1
    // whatever the earlier calls left)
    bfs_reset_kernel<<<grid_for_elems(J), 256, 0, st>>>(J, b.node, b.lh, b.order[b.cur], b.off[0], 1);
    count_launch();
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(J, kBfsTile), kBfsBlocks));
    bfs_level_launch<0>(tc, true, R, G, X, J, b.order[b.cur], b.node, b.lh, b.m, dv, b.flag, t, s.status, polls, st);
    int oi = 0;                  // off[oi]: the current level's slot ranges
    int64_t lb = 0, nl = 1;      // the level's first node and node count
    const int64_t levels = t.lfill_level;
    // the tail level moves samples at internal nodes of level lfill one level
    // down; a complete tree (every node of that level a leaf) has none
    const bool tail = t.node_count > t.nodes_upto_lfill;
    for (int64_t lvl = 0; lvl <= levels; lvl++) {
        const bool is_tail = lvl == levels;
        if (is_tail && !tail) break;
        if (is_tail)
            bfs_level_launch<2>(tc, false, R, G, X, J, b.order[b.cur], b.node, b.lh, b.m, dv, b.flag, t, s.status,
                                polls, st);
        else
            bfs_level_launch<1>(tc, J >= kTcrMinSlotsPerNode * nl, R, G, X, J, b.order[b.cur], b.node, b.lh, b.m, dv,
                                b.flag, t, s.status, polls, st);
        EXAFAC_TRY(scan_exclusive_u32_to_i64(b.flag, b.SL, J, b.SL + J, s.scan_sc, st));
        if (!is_tail) {
            bfs_offsets_kernel<<<grid_for_elems(nl), 256, 0, st>>>(nl, J, b.off[oi], b.SL, b.off[oi ^ 1]);
            count_launch();
        }
        bfs_scatter_kernel<<<grid_for_elems(J), 256, 0, st>>>(J, lb, nl, b.order[b.cur], b.node, b.off[oi], b.SL,
                                                             b.flag, b.order[b.cur ^ 1]);
        count_launch();
        b.cur ^= 1;
        oi ^= 1;
        lb = 2 * lb + 1;
        nl *= 2;
    }
    if (t.F > 1 && tc && t.F <= tc_layout(R, true).Rn) {
        const unsigned tblocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(J, kTcRows), 152));
        bfs_leaf_tc_kernel<<<tblocks, kTcThreads, bfs_leaf_tc_smem(R), st>>>(R, t, U, X, J, b.order[b.cur], b.node,
                                                                            b.lh, dv, s.N, col, s.samples, b.empty,
                                                                            s.status, polls);
    } else if (t.F > 1) {
        const size_t fsm = bfs_leaf_smem(R, (int)t.F);
        bfs_leaf_kernel<<<blocks, kBfsWarps * 32, fsm, st>>>(R, t, U, X, J, b.order[b.cur], b.node, b.lh, dv, s.N, col,
                                                            s.samples, b.empty);
    } else {
        bfs_leaf1_kernel<<<grid_for_elems(J), 256, 0, st>>>(t, J, b.node, s.N, col, s.samples, v_out);
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int sts_draw_bfs(Session& s, int n, int64_t J, const double* uni, cudaStream_t st) {
    const int N = s.N, R = s.R, Pf = packed_stride_f32(R);
    EXAFAC_CHECK_LAUNCH();
    BfsState& b = s.bfs;
    bfs_set_smem_limits();
    bfs_init_kernel<<<grid_for_elems(J * R), 256, 0, st>>>(R, J, b.h, b.empty);
    count_launch();
    for (int k = 0; k < N; k++) {
        if (k == n) continue;
        int nx = k + 1;
        if (nx == n) nx++;
        if (nx > N) nx = N;
        const float* Ek = s.EmatF + (int64_t)nx * R * R;
        // eigen tree of mode k, driven by h: v, then sh = h * E_next[v]
        EXAFAC_TRY(bfs_descend(s, s.etree, s.eigF + (int64_t)k * s.etree.node_count * Pf, nullptr, b.h,
                               uni + ((int64_t)k * 2 + 0) * J, J, n, b.v, st));
        bfs_scale_kernel<<<grid_for_elems(J * 32), 256, 0, st>>>(R, J, b.h, Ek, b.v, b.sh);
        count_launch();
        // row tree of mode k, driven by sh: the row, then h *= U_k[row]
        EXAFAC_TRY(bfs_descend(s, s.rtree[k], s.treeF[k], s.Uf[k], b.sh, uni + ((int64_t)k * 2 + 1) * J, J, k,
                               nullptr, st));
        bfs_row_update_kernel<<<grid_for_elems(J * 32), 256, 0, st>>>(R, J, s.Uf[k], s.samples, N, k, b.h);
        count_launch();
    }
    // h^T Phi h (one node: Phi), then the weights
    bfs_level_launch<0>(R >= kTcMinRank, true, R, s.PhiPF, b.h, J, b.order[b.cur], b.node, b.lh, b.m, nullptr, b.flag,
                        s.etree, s.status, s.wait_polls ? s.wait_polls : kSpinLimit, st);
    bfs_weight_kernel<<<grid_for_elems(J), 256, 0, st>>>(R, J, b.m, b.empty, s.weights);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

}  // namespace exafac

using namespace exafac;

extern "C" int exafac_quad_forms_f32(int32_t R, int64_t J, const float* X, const int64_t* node, const float* G,
                                     float* q, int32_t use_tc, void* stream) {
    EXAFAC_ARG(R >= 1 && R <= kMaxRank, "exafac_quad_forms_f32: R out of range");
    EXAFAC_ARG(J >= 1 && J <= INT32_MAX, "exafac_quad_forms_f32: J out of range");
    EXAFAC_ARG(X && node && G && q, "exafac_quad_forms_f32: null pointer");
    EXAFAC_ARG(use_tc >= 0 && use_tc <= 2, "exafac_quad_forms_f32: use_tc must be 0, 1 or 2");
    EXAFAC_ARG(!use_tc || R >= kTcMinRank, "exafac_quad_forms_f32: the tensor-core form needs R >= 32");
    bfs_set_smem_limits();
    TreeShape t{};
    bfs_level_launch<3>(use_tc != 0, use_tc == 2, R, G, X, J, nullptr, const_cast<int64_t*>(node), nullptr, q, nullptr,
                        nullptr, t, nullptr, kSpinLimit, (cudaStream_t)stream);
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}
