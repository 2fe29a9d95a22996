// PartitionTree build and PTSample kernels (partition_tree.hpp:117-380).
#include "tree.cuh"
#include "umma.cuh"

namespace exafac {

// Leaf Grams: one warp per leaf; the leaf's rows are staged in shared memory
// and each lane owns a strided set of packed entries, summing over rows in
// row order.
__global__ void tree_leaf_gram_kernel(TreeShape t, int R, const double* __restrict__ U, double* __restrict__ G) {
    extern __shared__ unsigned char smraw[];
    const int P = packed_size(R);
    const int warps = blockDim.x / 32;
    unsigned short* pa = reinterpret_cast<unsigned short*>(smraw);
    unsigned short* pb = pa + P;
    double* ublk = reinterpret_cast<double*>(smraw + align_up(2 * P * sizeof(unsigned short), 16));
    block_build_pairs(R, pa, pb);
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* u = ublk + (size_t)w * t.F * R;
    const int64_t first_leaf = t.node_count - t.leaf_count;
    for (int64_t li = (int64_t)blockIdx.x * warps + w; li < t.leaf_count; li += (int64_t)gridDim.x * warps) {
        const int64_t c = first_leaf + li;
        const int64_t leaf = tree_leaf_idx(t, c);
        const int64_t rows = (t.n - leaf * t.F) < t.F ? (t.n - leaf * t.F) : t.F;
        for (int64_t e = lane; e < rows * R; e += 32) u[e] = U[leaf * t.F * R + e];
        __syncwarp();
        double* g = G + c * P;
        for (int e = lane; e < P; e += 32) {
            const int a = pa[e], b = pb[e];
            double acc = 0.0;
            for (int64_t r = 0; r < rows; r++) acc = fma(u[r * R + a], u[r * R + b], acc);
            g[e] = acc;
        }
        __syncwarp();
    }
}

// Leaf Grams of the mixed forms, from the FP32 copy of the factor: a block
// per leaf (its rows staged in shared memory), a thread per packed entry
// (a, b).  Each product u_a u_b is split exactly into its FP32 rounding p and
// error fma(u_a, u_b, -p), and both are added into a compensated (hi, lo)
// FP32 sum (Knuth's two-sum), so the leaf sum carries about 48 bits on the
// FP32 pipe; it is widened to FP64 for the tree, whose internal sums are
// FP64.
__global__ void tree_leaf_gram_f32_kernel(TreeShape t, int R, const float* __restrict__ U, double* __restrict__ G) {
    extern __shared__ __align__(16) float lsm[];  // F x R
    const int P = packed_size(R);
    const int64_t first_leaf = t.node_count - t.leaf_count;
    for (int64_t li = blockIdx.x; li < t.leaf_count; li += gridDim.x) {
        const int64_t c = first_leaf + li;
        const int64_t leaf = tree_leaf_idx(t, c);
        const int64_t rows = (t.n - leaf * t.F) < t.F ? (t.n - leaf * t.F) : t.F;
        __syncthreads();
        for (int64_t e = threadIdx.x; e < rows * R; e += blockDim.x) lsm[e] = U[leaf * t.F * R + e];
        __syncthreads();
        double* g = G + c * P;
        for (int a = 0, base = 0; a < R; base += R - a, a++) {
            for (int b = a + threadIdx.x; b < R; b += blockDim.x) {
                float hi = 0.0f, lo = 0.0f;
                for (int64_t r = 0; r < rows; r++) {
                    const float x = lsm[r * R + a], y = lsm[r * R + b];
                    const float p = x * y;
                    const float err = __fmaf_rn(x, y, -p);
                    const float sum = hi + p;
                    const float bp = sum - hi;
                    lo += (hi - (sum - bp)) + (p - bp) + err;
                    hi = sum;
                }
                g[base + (b - a)] = (double)hi + (double)lo;
            }
        }
    }
}

// Leaf Grams of the mixed forms on the tensor cores (32 <= R <= 128, F <=
// 128): a block per leaf in turn, G_leaf = U_leaf^T U_leaf as one tcgen05.mma
// product whose A and B operands are the same staged tile, row a = component
// a over the leaf's rows (K-major: element (a, r) = U[leaf F + r][a], rows a
// >= R and r >= the leaf's rows zero), split into TF32 hi + lo parts:
// G ~ A_hi A_hi^T + A_hi A_lo^T + A_lo A_hi^T (relative error ~2^-21 of
// |U|^T |U|, FP32 accumulation in tensor memory).  The mixed forms use the
// tree only through its FP32 copy, so this accuracy is what they keep.  Warps
// read back their TMEM lanes (row a) and write the packed upper triangle as
// FP64 for the tree's FP64 internal sums.  The MMA barrier's waits are
// bounded as in the descents.
constexpr int kLeafTcThreads = 256;

__global__ void __launch_bounds__(kLeafTcThreads, 1)
    tree_leaf_gram_tc_kernel(TreeShape t, int R, const float* __restrict__ U, double* __restrict__ G,
                             DeviceStatus* status, uint32_t polls) {
    extern __shared__ __align__(16) unsigned char lg_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int F = (int)t.F;
    const int Rn = (R + 15) & ~15, Fk = (F + 15) & ~15;
    const uint32_t ncols = Rn <= 32 ? 32u : (Rn <= 64 ? 64u : 128u);
    const uint32_t sbo = (uint32_t)Fk * 32u;     // 8-row groups of the 128 x Fk tile
    const uint32_t tile_bytes = 128u * sbo / 8u;  // 128 x Fk x 4
    unsigned char* Ahi = lg_raw + ((1024u - (smem_u32(lg_raw) & 1023u)) & 1023u);
    unsigned char* Alo = Ahi + tile_bytes;
    if (w == 0) tmem_alloc(&tmem_base, ncols);
    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = umma_idesc_tf32(128, Rn);
    uint32_t phase = 0;
    const int P = packed_size(R);
    const int64_t first_leaf = t.node_count - t.leaf_count;
    for (int64_t li = blockIdx.x; li < t.leaf_count; li += gridDim.x) {
        const int64_t c = first_leaf + li;
        const int64_t leaf = tree_leaf_idx(t, c);
        const int rows = (int)((t.n - leaf * t.F) < t.F ? (t.n - leaf * t.F) : t.F);
        const float* Ub = U + leaf * t.F * R;
        __syncthreads();  // the previous leaf's MMAs and read-back are done with the tile
        // element (a, r .. r + 3): lanes over a (coalesced loads of a row,
        // 16-byte stores 16 bytes apart)
        const int total = 128 * (Fk / 4);
        for (int e = tid; e < total; e += kLeafTcThreads) {
            const int a = e & 127, r0 = 4 * (e >> 7);
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) v[q] = (a < R && r0 + q < rows) ? __ldg(Ub + (int64_t)(r0 + q) * R + a) : 0.0f;
            float4 h, l;
            h.x = tf32_rna(v[0]);
            h.y = tf32_rna(v[1]);
            h.z = tf32_rna(v[2]);
            h.w = tf32_rna(v[3]);
            l.x = tf32_rna(v[0] - h.x);
            l.y = tf32_rna(v[1] - h.y);
            l.z = tf32_rna(v[2] - h.z);
            l.w = tf32_rna(v[3] - h.w);
            const uint32_t off = (uint32_t)(a >> 3) * sbo + (uint32_t)(r0 >> 2) * 128u + (uint32_t)(a & 7) * 16u;
            *reinterpret_cast<float4*>(Ahi + off) = h;
            *reinterpret_cast<float4*>(Alo + off) = l;
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            for (int s = 0; s < Fk / 8; s++) {
                const uint32_t off = (uint32_t)s * 256u;
                const uint64_t dh = umma_desc(Ahi + off, 128u, sbo), dl = umma_desc(Alo + off, 128u, sbo);
                umma_tf32(tmem, dh, dh, idesc, s > 0 ? 1u : 0u);
                umma_tf32(tmem, dh, dl, idesc, 1u);
                umma_tf32(tmem, dl, dh, idesc, 1u);
            }
            umma_commit(&bar);
        }
        if (!mbar_wait_limited(&bar, phase, polls)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
        phase ^= 1u;
        tc_fence_after();
        {
            // warp w: lanes 32 (w % 4) .. + 31 = rows a; column blocks of 16
            // alternate between the two warp halves
            const int qw = w & 3, half = w >> 2;
            const int a = qw * 32 + lane;
            double* g = G + c * P;
            for (int cb = half; cb < Rn / 16; cb += 2) {
                float y[16];
                tmem_ld16(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(cb * 16), y);
                if (a < R) {
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const int b = cb * 16 + q;
                        if (b >= a && b < R) g[packed_index(R, a, b)] = (double)y[q];
                    }
                }
            }
        }
        tc_fence_before();
    }
    if (abort_flag) {
        if (tid == 0) report(status, EXAFAC_ERR_TIMEOUT, 22, blockIdx.x, 0);
        mbar_wait_limited(&bar, phase, polls);
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

// One level of internal nodes: G[c] = G[2c+1] + G[2c+2] (the reference adds
// both children to a zeroed node: 0 + (l + r) == l + r).
__global__ void tree_level_kernel(int64_t start, int64_t end, int P, double* __restrict__ G) {
    const int64_t total = (end - start) * P;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = start + i / P;
        int e = (int)(i % P);
        G[c * P + e] = G[(2 * c + 1) * P + e] + G[(2 * c + 2) * P + e];
    }
}

__global__ void tree_hadamard_kernel(int64_t nodes, int R, double* __restrict__ G, const double* __restrict__ M) {
    const int P = packed_size(R);
    const int64_t total = nodes * P;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int e = (int)(i % P);
        // e -> (a, b): walk rows (R <= 128, cheap).
        int a = 0, rem = e;
        while (rem >= R - a) {
            rem -= R - a;
            a++;
        }
        int b = a + rem;
        G[i] *= M[a * R + b];
    }
}

// PTSample for J samples (FP64), one sample per group of G warps.
__global__ void tree_sample_kernel(TreeShape t, int R, int G, int S, const double* __restrict__ Gt,
                                   const double* __restrict__ U, int64_t J, const double* __restrict__ x,
                                   double* __restrict__ hmul, const double* __restrict__ draws,
                                   uint32_t* __restrict__ out, int64_t out_stride) {
    extern __shared__ __align__(16) unsigned char tsdyn[];
    double *xs, *unused, *q;
    int gi;
    const SampleGroup<double> grp = sample_group<double>(tsdyn, R, G, xs, unused, q, gi);
    for (int64_t i = (int64_t)blockIdx.x * S + gi; i < J; i += (int64_t)gridDim.x * S) {
        for (int r = grp.tg; r < R; r += grp.nthreads()) xs[r] = x[i * R + r];
        grp.sync();
        grp.build_z(R, xs);
        const int64_t row = descend<double>(grp, t, R, Gt, U, xs, q, draws[i]);
        if (grp.tg == 0) out[i * out_stride] = (uint32_t)row;
        for (int r = grp.tg; r < R; r += grp.nthreads()) hmul[i * R + r] *= U[row * R + r];
        grp.sync();
    }
}

static int grid_for(int64_t work, int threads) {
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

int launch_tree_build(const TreeShape& t, int R, const double* U, double* G, cudaStream_t stream) {
    const int P = packed_size(R);
    int warps = 4;
    while (warps > 1 && sizeof(double) * warps * t.F * R > 160 * 1024) warps /= 2;
    size_t smem = align_up(2 * P * sizeof(unsigned short), 16) + sizeof(double) * warps * t.F * R;
    if (smem > 48 * 1024) {
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(tree_leaf_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    int blocks = (int)std::min<int64_t>((t.leaf_count + warps - 1) / warps, 152 * 8);
    tree_leaf_gram_kernel<<<blocks, warps * 32, smem, stream>>>(t, R, U, G); count_launch();
    EXAFAC_CHECK_LAUNCH();
    int64_t start = t.nodes_before_lfill, end = t.node_count - t.leaf_count;
    for (int64_t lvl = t.lfill_level; lvl >= 0; lvl--) {
        if (end > start) {
            tree_level_kernel<<<grid_for((end - start) * P, 256), 256, 0, stream>>>(start, end, P, G); count_launch();
            EXAFAC_CHECK_LAUNCH();
        }
        end = start;
        start = ((start + 1) / 2) - 1;
    }
    return EXAFAC_OK;
}

int launch_tree_build_f32(const TreeShape& t, int R, const float* U, double* G, DeviceStatus* status, uint32_t polls,
                          cudaStream_t stream) {
    const int P = packed_size(R);
    if (R >= 32 && t.F > 1 && t.F <= 128) {
        const size_t smem = 2 * sizeof(float) * 128 * (size_t)((t.F + 15) & ~15) + 1024;
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(tree_leaf_gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int blocks = (int)std::min<int64_t>(t.leaf_count, 152);
        tree_leaf_gram_tc_kernel<<<blocks, kLeafTcThreads, smem, stream>>>(t, R, U, G, status, polls);
    } else {
        const size_t smem = sizeof(float) * t.F * R;
        if (smem > 48 * 1024)
            EXAFAC_CUDA_TRY(
                cudaFuncSetAttribute(tree_leaf_gram_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int blocks = (int)std::min<int64_t>(t.leaf_count, 152 * 4);
        tree_leaf_gram_f32_kernel<<<blocks, 128, smem, stream>>>(t, R, U, G);
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    int64_t start = t.nodes_before_lfill, end = t.node_count - t.leaf_count;
    for (int64_t lvl = t.lfill_level; lvl >= 0; lvl--) {
        if (end > start) {
            tree_level_kernel<<<grid_for((end - start) * P, 256), 256, 0, stream>>>(start, end, P, G);
            count_launch();
            EXAFAC_CHECK_LAUNCH();
        }
        end = start;
        start = ((start + 1) / 2) - 1;
    }
    return EXAFAC_OK;
}

int launch_tree_hadamard(const TreeShape& t, int R, double* G, const double* M, cudaStream_t stream) {
    tree_hadamard_kernel<<<grid_for(t.node_count * packed_size(R), 256), 256, 0, stream>>>(t.node_count, R, G, M); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int launch_tree_sample(const TreeShape& t, int R, const double* G, const double* U, int64_t J, const double* x,
                       double* hmul, const double* draws, uint32_t* out, int64_t out_stride, cudaStream_t stream) {
    int Gw, S;
    sample_group_shape(R, sizeof(double), Gw, S);
    const size_t smem = (size_t)S * sample_group_bytes(R, sizeof(double));
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(tree_sample_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t blocks = (J + S - 1) / S;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    tree_sample_kernel<<<(int)blocks, S * Gw * 32, smem, stream>>>(t, R, Gw, S, G, U, J, x, hmul, draws, out,
                                                                   out_stride);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

}  // namespace exafac

using namespace exafac;

extern "C" int64_t exafac_tree_node_count(int64_t n, int32_t F) {
    if (n < 1 || F < 1) return 0;
    return make_tree_shape(n, F).node_count;
}

extern "C" int exafac_tree_build(int64_t n, int32_t F, int32_t R, const double* U, double* G, void* stream) {
    EXAFAC_ARG(n >= 1 && F >= 1 && R >= 1 && R <= kMaxRank, "exafac_tree_build: bad shape");
    EXAFAC_ARG(U && G, "exafac_tree_build: null pointer");
    return launch_tree_build(make_tree_shape(n, F), R, U, G, (cudaStream_t)stream);
}

extern "C" int exafac_tree_build_f32(int64_t n, int32_t F, int32_t R, const float* U, double* G, void* stream) {
    EXAFAC_ARG(n >= 1 && F >= 1 && R >= 1 && R <= kMaxRank, "exafac_tree_build_f32: bad shape");
    EXAFAC_ARG(U && G, "exafac_tree_build_f32: null pointer");
    return launch_tree_build_f32(make_tree_shape(n, F), R, U, G, nullptr, kSpinLimit, (cudaStream_t)stream);
}

extern "C" int exafac_tree_sample(int64_t n, int32_t F, int32_t R, const double* G, const double* U, int64_t J,
                                  const double* x, double* hmul, const double* draws, uint32_t* rows_out,
                                  int64_t rows_stride, void* stream) {
    EXAFAC_ARG(n >= 1 && F >= 1 && R >= 1 && R <= kMaxRank && J >= 0, "exafac_tree_sample: bad shape");
    if (F > kMaxLeafRows) {
        set_error("exafac_tree_sample: leaves of more than 128 rows are not supported");
        return EXAFAC_ERR_UNSUPPORTED;
    }
    EXAFAC_ARG(G && U && x && hmul && draws && rows_out, "exafac_tree_sample: null pointer");
    if (J == 0) return EXAFAC_OK;
    return launch_tree_sample(make_tree_shape(n, F), R, G, U, J, x, hmul, draws, rows_out, rows_stride,
                              (cudaStream_t)stream);
}
