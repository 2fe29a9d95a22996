// Segment tree of R x R Grams over F-row leaves (PartitionTree,
// partition_tree.hpp:48-380), GB300 layout: node c holds the packed upper
// triangle of its Gram, P = R(R+1)/2 doubles, row-major packed
// (entry (a, b), a <= b, at a*R - a*(a-1)/2 + (b - a)).
#pragma once
#include <algorithm>

#include "common.cuh"

namespace exafac {

struct TreeShape {
    int64_t n, F;
    int64_t leaf_count, node_count;
    int64_t lfill_level, lfill_count;
    int64_t nodes_upto_lfill, nodes_before_lfill, complete_level_offset;
};

// partition_tree.hpp:82-102 (log2_round_down: common.h:681-693).
inline TreeShape make_tree_shape(int64_t n, int64_t F) {
    TreeShape t;
    t.n = n;
    t.F = F;
    t.leaf_count = (n + F - 1) / F;
    t.node_count = 2 * t.leaf_count - 1;
    t.lfill_level = 0;
    t.lfill_count = 1;
    while (t.lfill_count * 2 <= t.leaf_count) {
        t.lfill_level++;
        t.lfill_count *= 2;
    }
    t.nodes_upto_lfill = t.lfill_count * 2 - 1;
    t.nodes_before_lfill = t.lfill_count - 1;
    t.complete_level_offset = t.nodes_before_lfill - (t.node_count - t.nodes_upto_lfill) / 2;
    return t;
}

__host__ __device__ __forceinline__ int64_t tree_leaf_idx(const TreeShape& t, int64_t c) {
    return c >= t.nodes_upto_lfill ? c - t.nodes_upto_lfill : c - t.complete_level_offset;
}
__host__ __device__ __forceinline__ bool tree_is_leaf(const TreeShape& t, int64_t c) { return 2 * c + 1 >= t.node_count; }
__host__ __device__ __forceinline__ int packed_size(int R) { return R * (R + 1) / 2; }
// Node stride of the FP32 tree copies the mixed forms descend on: the packed
// size rounded up to a multiple of 4 floats (zero padded), so that every node
// starts on a 16-byte boundary and is read with 16-byte loads.
__host__ __device__ __forceinline__ int packed_stride_f32(int R) { return (packed_size(R) + 3) & ~3; }
__host__ __device__ __forceinline__ int packed_index(int R, int a, int b) { return a * R - a * (a - 1) / 2 + (b - a); }

// Builds the tree over U (n x R, row-major).  G: node_count * P doubles.
int launch_tree_build(const TreeShape& t, int R, const double* U, double* G, cudaStream_t stream);
// The same from an FP32 copy of U, internal sums in FP64; leaf Grams on the
// tensor cores in TF32 hi + lo parts for 32 <= R, F <= 128 (waits bounded by
// `polls`, a timeout recorded in *status), else as compensated FP32 sums of
// exactly split products (about 48 bits).
int launch_tree_build_f32(const TreeShape& t, int R, const float* U, double* G, DeviceStatus* status, uint32_t polls,
                          cudaStream_t stream);

// Multiplies every node elementwise by the symmetric matrix M (R x R full)
// (multiply_matrices_against_provided, partition_tree.hpp:176-187).
int launch_tree_hadamard(const TreeShape& t, int R, double* G, const double* M, cudaStream_t stream);

// PTSample for J samples (warp per sample).
int launch_tree_sample(const TreeShape& t, int R, const double* G, const double* U, int64_t J, const double* x,
                       double* hmul, const double* draws, uint32_t* out, int64_t out_stride, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Device pieces shared by PTSample and the fused STS-CP sampler, in FP64
// (T = double, the reference's arithmetic) or FP32 (the mixed forms, over
// FP32 copies of the trees and factors).  A group of G warps (32 G threads,
// G in {1, 2, 4}) draws one sample at a time.  Per descent the group forms
// z_e = w_e x_a x_b in shared memory (packed order, w = 1 on the diagonal and
// 2 above it), so that x^T G x = sum_e z_e G_e for every packed node G: each
// level is then one coalesced pass over the node, P / (32 G) multiply-adds
// per thread, and a group sum in a fixed order.  G > 1 splits one sample's
// levels over several warps at large R, where a warp's share of shared memory
// (z holds P = R (R + 1) / 2 values) would otherwise leave few warps per SM.
// With G > 1 the block is the group (barriers are __syncthreads()).
// ---------------------------------------------------------------------------

__device__ __forceinline__ double fmat(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmat(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Fills pa/pb (P entries each) with the (row, col) of each packed index.
__device__ __forceinline__ void block_build_pairs(int R, unsigned short* pa, unsigned short* pb) {
    for (int a = threadIdx.x; a < R; a += blockDim.x) {
        int base = packed_index(R, a, a);
        for (int b = a; b < R; b++) {
            pa[base + b - a] = (unsigned short)a;
            pb[base + b - a] = (unsigned short)b;
        }
    }
}

// Node stride of the trees a descent in T reads: packed (the reference's
// layout) in FP64, padded to 16 bytes in FP32.
template <typename T>
__host__ __device__ __forceinline__ int node_stride(int R);
template <>
__host__ __device__ __forceinline__ int node_stride<double>(int R) { return packed_size(R); }
template <>
__host__ __device__ __forceinline__ int node_stride<float>(int R) { return packed_stride_f32(R); }

template <typename T>
struct SampleGroup {
    int G;     // warps per sample
    int tg;    // thread index within the group
    T* z;      // node_stride<T>(R) values (zero past P)
    T* red;    // G partial sums
    __device__ __forceinline__ int nthreads() const { return 32 * G; }
    __device__ __forceinline__ void sync() const {
        if (G == 1) __syncwarp();
        else __syncthreads();
    }
    // The group's sum of v (every thread gets it); partial sums of the warps
    // added in warp order.
    __device__ __forceinline__ T sum(T v) const {
        v = warp_sum(v);
        if (G == 1) return v;
        if ((tg & 31) == 0) red[tg >> 5] = v;
        __syncthreads();
        T s = red[0];
        for (int w = 1; w < G; w++) s += red[w];
        __syncthreads();
        return s;
    }
    // z = packed w_ab x_a x_b (rows split over the group's threads).
    __device__ __forceinline__ void build_z(int R, const T* x) const {
        for (int a = tg; a < R; a += nthreads()) {
            const T xa = x[a];
            const T xa2 = xa + xa;
            T* zr = z + packed_index(R, a, a) - a;
            zr[a] = xa * xa;
            for (int b = a + 1; b < R; b++) zr[b] = xa2 * x[b];
        }
        sync();
    }
    // x^T G x = sum_e z_e G_e for one node (ps = node_stride<T>(R) values).
    __device__ __forceinline__ T quad(int ps, const T* __restrict__ g) const;
};

// FP64: scalar loads, eight in flight per thread.
template <>
__device__ __forceinline__ double SampleGroup<double>::quad(int ps, const double* __restrict__ g) const {
    double a[8];
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = 0.0;
    const int step = nthreads();
    int e = tg;
    for (; e + 7 * step < ps; e += 8 * step) {
        double gv[8];
#pragma unroll
        for (int i = 0; i < 8; i++) gv[i] = __ldg(g + e + i * step);
#pragma unroll
        for (int i = 0; i < 8; i++) a[i] = fmat(z[e + i * step], gv[i], a[i]);
    }
    for (; e < ps; e += step) a[0] = fmat(z[e], __ldg(g + e), a[0]);
    return sum(((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7])));
}

// FP32: 16-byte loads of the node and of z (both padded with zeros to
// a multiple of 4), four in flight per thread.
template <>
__device__ __forceinline__ float SampleGroup<float>::quad(int ps, const float* __restrict__ g) const {
    const float4* g4 = reinterpret_cast<const float4*>(g);
    const float4* z4 = reinterpret_cast<const float4*>(z);
    const int n4 = ps >> 2;
    float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int step = nthreads();
    int e = tg;
    for (; e + 3 * step < n4; e += 4 * step) {
        float4 gv[4];
#pragma unroll
        for (int i = 0; i < 4; i++) gv[i] = __ldg(g4 + e + i * step);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const float4 zv = z4[e + i * step];
            a[i] = fmat(zv.x, gv[i].x, a[i]);
            a[i] = fmat(zv.y, gv[i].y, a[i]);
            a[i] = fmat(zv.z, gv[i].z, a[i]);
            a[i] = fmat(zv.w, gv[i].w, a[i]);
        }
    }
    for (; e < n4; e += step) {
        const float4 gv = __ldg(g4 + e), zv = z4[e];
        a[0] = fmat(zv.x, gv.x, a[0]);
        a[0] = fmat(zv.y, gv.y, a[0]);
        a[0] = fmat(zv.z, gv.z, a[0]);
        a[0] = fmat(zv.w, gv.w, a[0]);
    }
    return sum((a[0] + a[1]) + (a[2] + a[3]));
}

// One descent of PTSample (partition_tree.hpp:204-380) by the group, with
// the uniform d and z built from the descent vector x: root mass, one
// left-child quadratic form per level (cutoff = low + m_L / m), the tail
// level, then, for F > 1, the leaf's rows by the prefix of their squared dots
// U_j . x (thread per row; the prefix a warp scan in row order): the first
// row j < F - 1 with frac < prefix_j / total, else the leaf's last row.
// q: F values of group scratch.  Returns the chosen row (< n).
//
// A leaf whose rows all have zero dot with x (possible only through rounding
// of the cutoffs, in practice in FP32: the descent stepped into a child of
// zero mass) sets *empty and returns its first row; the caller gives the
// sample weight 0.  The reference's loop would pick the leaf's last slot
// there (0 / 0 comparisons), possibly past the tensor.
template <typename T>
__device__ __forceinline__ int64_t descend(const SampleGroup<T>& grp, const TreeShape& t, int R,
                                           const T* __restrict__ G, const T* __restrict__ U, const T* x, T* q, T d,
                                           bool* empty = nullptr) {
    const int P = node_stride<T>(R);  // node stride of G
    int64_t c = 0;
    T low = T(0), high = T(1);
    const T m = grp.quad(P, G);
    for (int64_t lvl = 0; lvl < t.lfill_level; lvl++) {
        const T mL = grp.quad(P, G + (2 * c + 1) * P);
        const T cutoff = low + mL / m;
        if (d <= cutoff) {
            c = 2 * c + 1;
            high = cutoff;
        } else {
            c = 2 * c + 2;
            low = cutoff;
        }
    }
    if (t.node_count > t.nodes_before_lfill && !tree_is_leaf(t, c)) {
        const T mL = grp.quad(P, G + (2 * c + 1) * P);
        const T cutoff = low + mL / m;
        if (d <= cutoff) {
            c = 2 * c + 1;
            high = cutoff;
        } else {
            c = 2 * c + 2;
            low = cutoff;
        }
    }
    const int64_t leaf = tree_leaf_idx(t, c);
    if (t.F <= 1) return leaf * t.F;
    const T frac = (d - low) / (high - low);
    const int64_t F = t.F;
    const int64_t rows = (t.n - leaf * F) < F ? (t.n - leaf * F) : F;
    const T* Ub = U + leaf * F * R;
    for (int64_t j = grp.tg; j < F; j += grp.nthreads()) {
        T v = T(0);
        if (j < rows) {
            const T* u = Ub + j * R;
            for (int r = 0; r < R; r++) v = fmat(__ldg(u + r), x[r], v);
        }
        q[j] = v * v;
    }
    grp.sync();
    // warp 0: inclusive prefix in row order (F <= 128), then the first row
    // with frac < prefix / total
    int64_t res = 0;
    bool is_empty = false;
    if (grp.tg < 32) {
        const int lane = grp.tg;
        T incl[4];
        T carry = T(0);
#pragma unroll
        for (int blk = 0; blk < 4; blk++) {
            const int64_t j = 32 * blk + lane;
            T v = j < F ? q[j] : T(0);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const T u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            incl[blk] = carry + v;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
        const T total = carry;
        if (!(total > T(0))) {
            is_empty = true;
        } else {
            res = F - 1;
#pragma unroll
            for (int blk = 0; blk < 4; blk++) {
                const int64_t j = 32 * blk + lane;
                const bool hit = (j < F - 1) && (frac < incl[blk] / total);
                const unsigned mask = __ballot_sync(0xffffffffu, hit);
                if (mask) {
                    res = 32 * blk + __ffs(mask) - 1;
                    break;
                }
            }
            // frac >= 1 (the uniform equal to the leaf's upper cutoff) leaves
            // the last slot, which a partial leaf does not hold
            if (res >= rows) res = rows - 1;
        }
    }
    if (grp.G > 1) {  // broadcast warp 0's choice to the other warps (through q, read by now)
        // (a 32-bit slot: q is only 4-byte aligned in the FP32 layout; res < 128)
        __syncthreads();
        if (grp.tg == 0) reinterpret_cast<int*>(q)[0] = is_empty ? -1 : (int)res;
        __syncthreads();
        const int v = reinterpret_cast<const int*>(q)[0];
        is_empty = v < 0;
        res = is_empty ? 0 : (int64_t)v;
        __syncthreads();
    }
    if (is_empty) {
        if (empty) *empty = true;
        return leaf * F;
    }
    return res + leaf * F;
}

// Leaves of at most this many rows (PTSample's F); the STS-CP row trees use
// F = R <= 128.
constexpr int kMaxLeafRows = 128;

// Shared memory of one sample's group: z (the node stride: P in FP64, P
// rounded up to 4 in FP32), h and sh (R each), q (128), red (8), in elements
// of esz bytes, rounded to 16 bytes.
__host__ __device__ inline size_t sample_group_bytes(int R, int esz) {
    const int ps = esz == 4 ? packed_stride_f32(R) : packed_size(R);
    return ((size_t)esz * (ps + 2 * R + kMaxLeafRows + 8) + 15) / 16 * 16;
}

// Warps per sample (G) and samples per block (S) for rank R and element size
// esz: G = 4 above P = 4096 (R > 90), 2 above P = 1024 (R > 44), else 1; with
// G = 1 up to 8 samples (warps) per block, fewer when their shared memory
// would pass 64 KB.
inline void sample_group_shape(int R, int esz, int& G, int& S) {
    const int P = packed_size(R);
    G = P > 4096 ? 4 : (P > 1024 ? 2 : 1);
    S = 1;
    if (G == 1) S = (int)std::max<size_t>(1, std::min<size_t>(8, (64 * 1024) / sample_group_bytes(R, esz)));
}

// The calling thread's group, and its h / sh / q buffers, in dynamic shared
// memory laid out group after group.
template <typename T>
__device__ __forceinline__ SampleGroup<T> sample_group(unsigned char* dyn, int R, int G, T*& h, T*& sh, T*& q,
                                                       int& gi) {
    const size_t bytes = sample_group_bytes(R, sizeof(T));
    gi = (threadIdx.x >> 5) / G;
    T* base = reinterpret_cast<T*>(dyn + gi * bytes);
    const int P = node_stride<T>(R);
    h = base + P;
    sh = h + R;
    q = sh + R;
    SampleGroup<T> grp;
    grp.G = G;
    grp.tg = threadIdx.x - gi * 32 * G;
    grp.z = base;
    grp.red = q + kMaxLeafRows;
    // z past the packed entries stays zero (build_z writes entries < P only)
    for (int e = packed_size(R) + grp.tg; e < P; e += grp.nthreads()) base[e] = T(0);
    return grp;
}

}  // namespace exafac
