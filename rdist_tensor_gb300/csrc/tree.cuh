// Segment tree of R x R Grams over F-row leaves (PartitionTree,
// partition_tree.hpp:48-380), GB300 layout: node c holds the packed upper
// triangle of its Gram, P = R(R+1)/2 doubles, row-major packed
// (entry (a, b), a <= b, at a*R - a*(a-1)/2 + (b - a)).
#pragma once
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
__host__ __device__ __forceinline__ int packed_index(int R, int a, int b) { return a * R - a * (a - 1) / 2 + (b - a); }

// Builds the tree over U (n x R, row-major).  G: node_count * P doubles.
int launch_tree_build(const TreeShape& t, int R, const double* U, double* G, cudaStream_t stream);

// Multiplies every node elementwise by the symmetric matrix M (R x R full)
// (multiply_matrices_against_provided, partition_tree.hpp:176-187).
int launch_tree_hadamard(const TreeShape& t, int R, double* G, const double* M, cudaStream_t stream);

// PTSample for J samples (warp per sample).
int launch_tree_sample(const TreeShape& t, int R, const double* G, const double* U, int64_t J, const double* x,
                       double* hmul, const double* draws, uint32_t* out, int64_t out_stride, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Device pieces shared with the fused STS-CP sampler.
// ---------------------------------------------------------------------------

// Per-warp precomputation of z_e = w_e x_a x_b (w = 1 on the diagonal, 2 off
// it) so that x^T G x = sum_e z_e G_e for every packed node G.
__device__ __forceinline__ void warp_build_z(int R, const double* x_sm, const unsigned short* pa,
                                             const unsigned short* pb, double* z_sm) {
    const int P = packed_size(R);
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < P; e += 32) {
        int a = pa[e], b = pb[e];
        double v = x_sm[a] * x_sm[b];
        z_sm[e] = (a == b) ? v : 2.0 * v;
    }
    __syncwarp();
}

__device__ __forceinline__ double warp_quad(int R, const double* z_sm, const double* __restrict__ g) {
    const int P = packed_size(R);
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int e = lane; e < P; e += 32) acc = fma(z_sm[e], __ldg(g + e), acc);
    return warp_sum(acc);
}

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

// One descent of PTSample (partition_tree.hpp:226-380) by the calling warp.
// z_sm: the sample's z (see warp_build_z); x_sm: the descent vector x (R);
// q_sm: F doubles of scratch.  Returns the chosen row (< n unless the
// uniform hits the upper edge of a partial leaf, see the reference).
__device__ __forceinline__ int64_t warp_descend(const TreeShape& t, int R, const double* __restrict__ G,
                                                const double* __restrict__ U, const double* z_sm, const double* x_sm,
                                                double* q_sm, double d) {
    const int P = packed_size(R);
    const int lane = threadIdx.x & 31;
    int64_t c = 0;
    double low = 0.0, high = 1.0;
    const double m = warp_quad(R, z_sm, G);
    for (int64_t lvl = 0; lvl < t.lfill_level; lvl++) {
        double mL = warp_quad(R, z_sm, G + (2 * c + 1) * P);
        double cutoff = low + mL / m;
        if (d <= cutoff) {
            c = 2 * c + 1;
            high = cutoff;
        } else {
            c = 2 * c + 2;
            low = cutoff;
        }
    }
    if (t.node_count > t.nodes_before_lfill && !tree_is_leaf(t, c)) {
        double mL = warp_quad(R, z_sm, G + (2 * c + 1) * P);
        double cutoff = low + mL / m;
        if (d <= cutoff) {
            c = 2 * c + 1;
            high = cutoff;
        } else {
            c = 2 * c + 2;
            low = cutoff;
        }
    }
    const int64_t leaf = tree_leaf_idx(t, c);
    int64_t res = 0;
    if (t.F > 1) {
        const double frac = (d - low) / (high - low);
        const int64_t F = t.F;
        const int64_t rows = (t.n - leaf * F) < F ? (t.n - leaf * F) : F;
        for (int64_t j = lane; j < F; j += 32) {
            double v = 0.0;
            if (j < rows) {
                const double* u = U + (leaf * F + j) * R;
                for (int r = 0; r < R; r++) v = fma(__ldg(u + r), x_sm[r], v);
            }
            q_sm[j] = v * v;
        }
        __syncwarp();
        // Sequential exclusive prefix of q^2 in row order, as the reference
        // accumulates it; q_sm[j] becomes the prefix through row j.
        double total = 0.0;
        if (lane == 0) {
            double run = 0.0;
            for (int64_t j = 0; j < F; j++) {
                run += q_sm[j];
                q_sm[j] = run;
            }
            total = run;
        }
        total = __shfl_sync(0xffffffffu, total, 0);
        __syncwarp();
        res = F - 1;
        for (int64_t base = 0; base < F - 1; base += 32) {
            int64_t j = base + lane;
            bool hit = (j < F - 1) && (frac < q_sm[j] / total);
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            if (mask) {
                res = base + __ffs(mask) - 1;
                break;
            }
        }
        __syncwarp();
    }
    return res + leaf * t.F;
}

}  // namespace exafac
