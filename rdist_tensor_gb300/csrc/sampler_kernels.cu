// Samplers on the GPU: the session's Philox stream, CP-ARLS-LEV (leverage
// scores, discrete CDF, inverse-CDF draws) and STS-CP (computeM, eigen trees,
// fused warp-per-sample descent through the eigen and row trees).
#include "dense.cuh"
#include "engine.cuh"
#include "prims.cuh"

namespace exafac {

// The stream counter lives in device memory (counters[kRngSlot]) and advances
// by one per call in a one-thread kernel, so a captured and replayed sweep
// draws fresh uniforms on every replay.
__global__ void philox_uniform_kernel(double* out, int64_t count, uint64_t seed, const int64_t* __restrict__ ctr_dev) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i = 2 * t;
    if (i >= count) return;
    const uint64_t ctr = (uint64_t)*ctr_dev;
    uint4 c = make_uint4((unsigned)t, (unsigned)(t >> 32), (unsigned)ctr, (unsigned)(ctr >> 32));
    uint4 r = philox4x32_10(c, make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    out[i] = u53(r.x, r.y);
    if (i + 1 < count) out[i + 1] = u53(r.z, r.w);
}

__global__ void philox_advance_kernel(int64_t* ctr_dev) { *ctr_dev += 1; }

int gen_uniforms(Session& s, double* out, int64_t count, cudaStream_t st) {
    if (count <= 0) return EXAFAC_OK;
    int64_t threads = (count + 1) / 2;
    int64_t* ctr = s.counters + kRngSlot;
    philox_uniform_kernel<<<(unsigned)ceil_div(threads, 256), 256, 0, st>>>(out, count, s.seed, ctr); count_launch();
    philox_advance_kernel<<<1, 1, 0, st>>>(ctr); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// ---------------------------------------------------------------------------
// CP-ARLS-LEV
// ---------------------------------------------------------------------------

// libstdc++ discrete_distribution::param_type::_M_initialize
// (bits/random.tcc:2657-2678) for short weight vectors, strictly in order:
// sequential sum, p_i = w_i / sum, sequential partial sums, last = 1.0.
// The weights are staged in shared memory (n <= kExactCdfMax) so the two
// serial loops run on shared-memory latency.
__global__ void cdf_sequential_kernel(const double* __restrict__ w, int64_t n, double* __restrict__ cdf,
                                      double* __restrict__ total, const uint32_t* __restrict__ gather,
                                      const int64_t* __restrict__ n_dev) {
    extern __shared__ double sh[];
    __shared__ double sum_sh;
    if (n_dev) n = min(n, *n_dev);
    if (n < 1) {
        if (threadIdx.x == 0) *total = 0.0;
        return;
    }
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) sh[i] = w[gather ? (int64_t)gather[i] : i];
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int64_t i = 0; i < n; i++) sum += sh[i];
        sum_sh = sum;
        *total = sum;
    }
    __syncthreads();
    const double sum = sum_sh;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) sh[i] = sh[i] / sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double run = 0.0;
        double next = sh[0];
        for (int64_t i = 0; i < n; i++) {
            const double cur = next;
            if (i + 1 < n) next = sh[i + 1];
            run += cur;
            sh[i] = run;
        }
        sh[n - 1] = 1.0;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) cdf[i] = sh[i];
}

// Guide table of a CDF (the bucket method of inverse-CDF sampling):
// guide[b] = lower_bound(cdf, b / B), b = 0..B.  For u in [b/B, (b+1)/B) the
// first entry >= u lies in [guide[b], guide[b+1]], because lower_bound is
// monotone in u and cdf[guide[b+1]] >= (b+1)/B > u.  B is a power of two, so
// b/B and floor(u B) are exact.
__global__ void cdf_guide_kernel(const double* __restrict__ cdf, int64_t n, uint32_t* __restrict__ guide,
                                 const int64_t* __restrict__ n_dev) {
    pdl_wait();
    pdl_trigger();
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > kGuideBuckets) return;
    if (n_dev) n = min(n, *n_dev);
    if (n < 1) {
        guide[b] = 0;
        return;
    }
    const double x = (double)b / (double)kGuideBuckets;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (cdf[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    guide[b] = (uint32_t)(lo < n ? lo : n - 1);
}

// CDF of mode k's leverage scores.  list == null: over all rows.  Otherwise
// over the rows in list[0 .. *count_dev) (ascending; the rows whose scores can
// be nonzero after a sampled update): the partial sums at those rows are the
// ones the full CDF takes there (the other rows add exactly zero), so a draw
// lands on the same row; only the final 1.0 sits at the last listed row.
// The listed rows' scores are read from scores_c, where the leverage kernels
// left them by list position (contiguous, no gather).
int arls_build_cdf(Session& s, int k, const uint32_t* list, const int64_t* count_dev, cudaStream_t st) {
    const double* w = list ? s.scores_c : s.scores[k];
    const int64_t n = s.dims[k];
    s.cdf_compact[k] = list != nullptr;
    if (n < 2) {
        // A one-row distribution always yields row 0 and consumes no draw.
        s.cdf_compact[k] = false;
        cdf_sequential_kernel<<<1, 32, sizeof(double) * n, st>>>(s.scores[k], n, s.cdf[k], s.cdf_total + k, nullptr,
                                                                  nullptr);
        count_launch();
        EXAFAC_CHECK_LAUNCH();
        return EXAFAC_OK;
    }
    if (n <= kExactCdfMax) {
        const size_t smem = sizeof(double) * n;
        if (smem > 48 * 1024)
            EXAFAC_CUDA_TRY(cudaFuncSetAttribute(cdf_sequential_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem));
        cdf_sequential_kernel<<<1, 256, smem, st>>>(w, n, s.cdf[k], s.cdf_total + k, nullptr, count_dev);
        count_launch();
    } else {
        EXAFAC_TRY(scan_cdf_f64(w, s.cdf[k], n, s.cdf_total + k, s.scan_sc, st, nullptr, count_dev));
    }
    EXAFAC_CUDA_TRY(launch_dependent(cdf_guide_kernel, (unsigned)ceil_div(kGuideBuckets + 1, 256), 256, 0, st,
                                     (const double*)s.cdf[k], n, s.guide[k], count_dev));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// compute_DAGAT (common.h:727-746) row by row: l_r = u_r^T P u_r with
// y = P u (dsymm) then the dot product.  Warp per row.
__global__ void leverage_kernel(int R, const double* __restrict__ U, const double* __restrict__ Pm, int64_t rows,
                                const uint32_t* __restrict__ list, const int64_t* __restrict__ count_dev,
                                double* __restrict__ scores, double* __restrict__ scores_c) {
    extern __shared__ double sm[];
    double* Psm = sm;
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* usm = Psm + R * R + w * R;
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) Psm[e] = Pm[e];
    __syncthreads();
    const int64_t cnt = list ? *count_dev : rows;
    for (int64_t i = (int64_t)blockIdx.x * warps + w; i < cnt; i += (int64_t)gridDim.x * warps) {
        const int64_t r = list ? (int64_t)list[i] : i;
        for (int a = lane; a < R; a += 32) usm[a] = U[r * R + a];
        __syncwarp();
        double acc = 0.0;
        for (int a = lane; a < R; a += 32) {
            double y = 0.0;
            for (int b = 0; b < R; b++) y = fma(Psm[a * R + b], usm[b], y);
            acc = fma(usm[a], y, acc);
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            scores[r] = acc;
            if (list) scores_c[i] = acc;  // by list position, for the CDF
        }
        __syncwarp();
    }
}

int arls_leverage(Session& s, int k, bool all_rows, const double* pinv, cudaStream_t st) {
    const int R = s.R;
    const int warps = 8;
    size_t smem = sizeof(double) * ((size_t)R * R + warps * R);
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(leverage_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t rows = all_rows ? s.dims[k] : s.dims[k];
    int blocks = (int)std::min<int64_t>(ceil_div(rows, warps), 152 * 16);
    leverage_kernel<<<blocks, warps * 32, smem, st>>>(R, s.F.U[k], pinv, s.dims[k], all_rows ? nullptr : s.touched,
                                                      s.counters + 2, s.scores[k], s.scores_c); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

struct ArlsModes {
    const double* cdf[kMaxModes];
    const double* scores[kMaxModes];
    const uint32_t* guide[kMaxModes];
    const uint32_t* rowmap[kMaxModes];  // compact CDF: entry -> row (null: entry = row)
    const int64_t* len[kMaxModes];      // compact CDF: its length on the device
    int64_t dims[kMaxModes];
};

// CP_ARLS_LEV::KRPDrawSamples + draw_leverage_score_samples
// (cp_arls_lev.hpp:36-163) at one rank, thread per sample: the draw is the
// first CDF entry >= u (lower_bound, searched between the guide entries of
// u's bucket).  The weight is the reference's exp(sum_k (log sum_k - log l_k)
// - log J) in the FP64 form (log_form != 0).  The mixed forms take the
// product (prod_k sum_k) / (J prod_k l_k) instead: the same number to ~1e-14
// relative (the rounding of the log-exp form itself), with one division in
// place of N logs and an exp, which on GB300's narrow FP64 pipe dominated the
// draw; a product that leaves the normal range (or a zero score) falls back
// to the log form.
__global__ void arls_draw_kernel(int N, int n, int64_t J, int log_form, ArlsModes m, const double* __restrict__ total,
                                 const double* __restrict__ uni, const uint32_t* __restrict__ perms,
                                 uint32_t* __restrict__ samples, double* __restrict__ weights,
                                 DeviceStatus* status) {
    __shared__ double log_total[kMaxModes];
    if (threadIdx.x < N) log_total[threadIdx.x] = log(total[threadIdx.x]);
    __syncthreads();
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J) return;
    double num = 1.0, den = (double)J;
    for (int k = 0; k < N; k++) {
        if (k == n) continue;
        const int64_t I = m.dims[k];
        int64_t src = perms ? (int64_t)perms[(int64_t)k * J + t] : t;
        if (src >= J) {
            report(status, EXAFAC_ERR_DEVICE, 3, src, J);
            src = t;
        }
        int64_t idx = 0;
        if (I >= 2) {
            const int64_t L = m.len[k] ? min(I, *m.len[k]) : I;  // CDF entries
            const double u = uni[(int64_t)k * J + src];
            if (L >= 1) {
                const double* cdf = m.cdf[k];
                const int b = min((int)(u * (double)kGuideBuckets), kGuideBuckets - 1);
                int64_t lo = m.guide[k][b], hi = min((int64_t)m.guide[k][b + 1] + 1, L);
                while (lo < hi) {
                    int64_t mid = (lo + hi) >> 1;
                    if (cdf[mid] < u) lo = mid + 1;
                    else hi = mid;
                }
                idx = lo < L ? lo : L - 1;
                if (m.rowmap[k]) idx = m.rowmap[k][idx];
                if (idx >= I) {  // a row list entry out of range: report, take row 0
                    report(status, EXAFAC_ERR_DEVICE, 7, idx, I);
                    idx = 0;
                }
            }
        }
        num *= total[k];
        den *= m.scores[k][idx];
        samples[t * N + k] = (uint32_t)idx;
    }
    samples[t * N + n] = 0;
    double w = log_form ? 0.0 : num / den;
    const uint32_t ew = (uint32_t)(__double_as_longlong(w) >> 52) & 0x7ffu;
    if (log_form || ew == 0 || ew == 0x7ffu) {  // the FP64 form, or zero, subnormal, inf or nan
        double lw = 0.0 - log((double)J);
        for (int k = 0; k < N; k++)
            if (k != n) lw += 0.0 + (log_total[k] - log(m.scores[k][samples[t * N + k]]));
        w = exp(lw);
    }
    weights[t] = w;
}

int arls_draw(Session& s, int n, int64_t J, const double* uni, const uint32_t* perms, cudaStream_t st) {
    ArlsModes m;
    for (int k = 0; k < kMaxModes; k++) {
        m.cdf[k] = k < s.N ? s.cdf[k] : nullptr;
        m.scores[k] = k < s.N ? s.scores[k] : nullptr;
        m.guide[k] = k < s.N ? s.guide[k] : nullptr;
        const bool compact = k < s.N && s.cdf_compact[k];
        m.rowmap[k] = compact ? s.nzrows[k] : nullptr;
        m.len[k] = compact ? s.nzcount + k : nullptr;
        m.dims[k] = k < s.N ? s.dims[k] : 0;
    }
    const int log_form = s.cfg.precision == EXAFAC_PREC_FP64;
    arls_draw_kernel<<<(unsigned)ceil_div(J, 256), 256, 0, st>>>(s.N, n, J, log_form, m, s.cdf_total, uni, perms, s.samples,
                                                                  s.weights, s.status); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// ---------------------------------------------------------------------------
// STS-CP
// ---------------------------------------------------------------------------

// FP32 copies (round to nearest even, in integer arithmetic) of FP64 arrays.
__global__ void narrow_copy_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = narrow_f64(in[i]);
}

static int narrow_copy(const double* in, float* out, int64_t n, cudaStream_t st) {
    if (n <= 0) return EXAFAC_OK;
    narrow_copy_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 16), 256, 0, st>>>(in, out, n);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// FP32 copies of packed nodes (P doubles each) at the padded FP32 node stride
// Pf, the padding zeroed.
__global__ void narrow_nodes_kernel(const double* __restrict__ in, int P, float* __restrict__ out, int Pf,
                                    int64_t nodes) {
    for (int64_t c = blockIdx.x; c < nodes; c += gridDim.x)  // a block per node, threads along it
        for (int e = threadIdx.x; e < Pf; e += blockDim.x) out[c * Pf + e] = e < P ? narrow_f64(in[c * P + e]) : 0.0f;
}

static int narrow_nodes(const double* in, float* out, int R, int64_t nodes, cudaStream_t st) {
    const int P = packed_size(R), Pf = packed_stride_f32(R);
    if (nodes <= 0) return EXAFAC_OK;
    narrow_nodes_kernel<<<(unsigned)std::min<int64_t>(nodes, 152 * 16), 256, 0, st>>>(in, P, out, Pf, nodes);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// STS_CP::computeM part 1 (sts_cp.hpp:81-102): suffix Hadamard products of
// the factor Grams over the modes != n; chain[n] is cleared.
__global__ void sts_chain_kernel(int N, int n, int R, const double* __restrict__ gram, double* __restrict__ chain) {
    const int R2 = R * R;
    for (int e = threadIdx.x; e < R2; e += blockDim.x) {
        double last = 1.0;
        for (int k = N - 1; k >= 0; k--) {
            if (k == n) {
                chain[(int64_t)k * R2 + e] = 0.0;
                continue;
            }
            last = gram[(int64_t)k * R2 + e] * last;
            chain[(int64_t)k * R2 + e] = last;
        }
    }
}

// computeM part 2 (sts_cp.hpp:118-153): W[:, R-1-v] = v-th eigenvector /
// sqrt(lambda_v) (dropped at lambda_v <= 1e-8), Phi = W W^T, the rows of W^T
// become E[N], and chain[k] *= Phi for k >= 1.
__global__ void sts_phi_kernel(int N, int n, int R, const double* __restrict__ V0, const double* __restrict__ L0,
                               double* __restrict__ chain, double* __restrict__ E, double* __restrict__ Phi,
                               double* __restrict__ PhiP) {
    extern __shared__ double W[];
    const int R2 = R * R;
    for (int e = threadIdx.x; e < R2; e += blockDim.x) {
        int u = e / R, v = e % R;
        double lam = L0[v];
        W[u * R + (R - 1 - v)] = lam > 1e-8 ? V0[u * R + v] / sqrt(lam) : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R2; e += blockDim.x) {
        int a = e / R, b = e % R;
        E[(int64_t)N * R2 + a * R + b] = W[b * R + a];
        double acc = 0.0;
        for (int v = 0; v < R; v++) acc = fma(W[a * R + v], W[b * R + v], acc);
        Phi[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R2; e += blockDim.x) {
        int a = e / R, b = e % R;
        double p = Phi[a <= b ? a * R + b : b * R + a];
        if (a <= b) PhiP[packed_index(R, a, b)] = p;
        for (int k = N - 1; k > 0; k--)
            if (k != n) chain[(int64_t)k * R2 + e] *= p;
    }
}

// computeM part 3 (sts_cp.hpp:156-176): E[k] row v = sqrt(lambda_v) * v-th
// eigenvector of chain[k] (k = 1..N-1, k != n).
__global__ void sts_emat_kernel(int N, int n, int R, const double* __restrict__ V, const double* __restrict__ L,
                                double* __restrict__ E) {
    const int R2 = R * R;
    for (int k = 1; k < N; k++) {
        if (k == n) continue;
        for (int e = threadIdx.x; e < R2; e += blockDim.x) {
            int v = e / R, u = e % R;
            E[(int64_t)k * R2 + v * R + u] = V[(int64_t)k * R2 + u * R + v] * sqrt(L[(int64_t)k * R + v]);
        }
    }
}

// Eigen tree of each sampled mode k (sts_cp.hpp:179-187): PartitionTree over
// the rows of E[next(k)] with one row per leaf, then every node times the
// Gram of U_k; the same operations in the same order as the reference (leaf
// outer products, pairwise sums bottom-up, then the Hadamard product), spread
// over the GPU: one launch for the leaves of every sampled mode, one per
// level for the sums, one for the products.

__device__ __forceinline__ int eigen_next(int N, int n, int k) {
    int nxt = k + 1;
    if (nxt == n) nxt++;
    return nxt > N ? N : nxt;
}

// The leaves' packed outer products: a warp per packed row a of one leaf of
// one sampled mode, its lanes along the row (b = a .. R - 1).
__global__ void eigen_leaves_kernel(int N, int n, int R, TreeShape t, const double* __restrict__ E,
                                    double* __restrict__ eigG) {
    const int P = packed_size(R);
    const int64_t first_leaf = t.node_count - t.leaf_count;
    const int64_t rows = (int64_t)N * t.leaf_count * R;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < rows; q += nw) {
        const int k = (int)(q / (t.leaf_count * R));
        if (k == n) continue;
        const int64_t rem = q - (int64_t)k * t.leaf_count * R;
        const int64_t li = rem / R;
        const int a = (int)(rem - li * R);
        const double* Ek = E + (int64_t)eigen_next(N, n, k) * R * R;
        const int64_t v = tree_leaf_idx(t, first_leaf + li);
        const double xa = Ek[v * R + a];
        double* out = eigG + ((int64_t)k * t.node_count + first_leaf + li) * P + packed_index(R, a, a);
        for (int b = a + lane; b < R; b += 32) out[b - a] = xa * Ek[v * R + b];
    }
}

// Internal nodes [start, end) of every sampled mode's tree: G[c] = G[2c+1] + G[2c+2].
__global__ void eigen_level_kernel(int N, int n, int P, TreeShape t, int64_t start, int64_t end,
                                   double* __restrict__ eigG) {
    const int64_t per_mode = (end - start) * P;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)N * per_mode;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(i / per_mode);
        if (k == n) continue;
        const int64_t c = start + (i % per_mode) / P;
        const int e = (int)(i % P);
        double* G = eigG + (int64_t)k * t.node_count * P;
        G[c * P + e] = G[(2 * c + 1) * P + e] + G[(2 * c + 2) * P + e];
    }
}

// Every node times its mode's Gram, elementwise: a warp per packed row a of
// one node of one sampled mode, its lanes along the row.
__global__ void eigen_hadamard_kernel(int N, int n, int R, TreeShape t, const double* __restrict__ gram,
                                      double* __restrict__ eigG) {
    const int P = packed_size(R);
    const int64_t rows = (int64_t)N * t.node_count * R;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < rows; q += nw) {
        const int k = (int)(q / (t.node_count * R));
        if (k == n) continue;
        const int64_t rem = q - (int64_t)k * t.node_count * R;
        const int64_t c = rem / R;
        const int a = (int)(rem - c * R);
        double* G = eigG + ((int64_t)k * t.node_count + c) * P + packed_index(R, a, a);
        const double* g = gram + (int64_t)k * R * R + (int64_t)a * R;
        for (int b = a + lane; b < R; b += 32) G[b - a] *= g[b];
    }
}

static int build_eigen_trees(Session& s, int n, cudaStream_t st) {
    const int N = s.N, R = s.R, P = s.P;
    const TreeShape& t = s.etree;
    auto grid = [](int64_t work) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(work, 256), 152 * 16)); };
    eigen_leaves_kernel<<<grid((int64_t)N * t.leaf_count * R * 32), 256, 0, st>>>(N, n, R, t, s.Emat, s.eigG);
    count_launch();
    int64_t start = t.nodes_before_lfill, end = t.node_count - t.leaf_count;
    for (int64_t lvl = t.lfill_level; lvl >= 0; lvl--) {
        if (end > start) {
            eigen_level_kernel<<<grid((int64_t)N * (end - start) * P), 256, 0, st>>>(N, n, P, t, start, end, s.eigG);
            count_launch();
        }
        end = start;
        start = ((start + 1) / 2) - 1;
    }
    eigen_hadamard_kernel<<<grid((int64_t)N * t.node_count * R * 32), 256, 0, st>>>(N, n, R, t, s.gram, s.eigG);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// The reference's factors: eigendecompositions of chain[first] (Phi, E[N])
// and of chain[k] (E[k]).
static int sts_eigen_factors(Session& s, int n, cudaStream_t st) {
    const int N = s.N, R = s.R, R2 = R * R;
    const int first = (n == 0) ? 1 : 0;
    EXAFAC_TRY(launch_syev(R, s.chain + (int64_t)first * R2, 0, 1, s.eigV, s.eigL, 0, nullptr, 0.0, s.vt, st));
    const size_t phi_smem = sizeof(double) * R2;
    if (phi_smem > 48 * 1024)
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(sts_phi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)phi_smem));
    sts_phi_kernel<<<1, 256, phi_smem, st>>>(N, n, R, s.eigV, s.eigL, s.chain, s.Emat, s.Phi, s.PhiP); count_launch();
    EXAFAC_CHECK_LAUNCH();
    if (N > 1) {
        // matrices 1..N-1 (chain[n] was cleared, its decomposition is trivial)
        EXAFAC_TRY(launch_syev(R, s.chain + R2, R2, N - 1, s.eigV + R2, s.eigL + R, R2, nullptr, 0.0, s.vt, st));
    }
    sts_emat_kernel<<<1, 256, 0, st>>>(N, n, R, s.eigV, s.eigL, s.Emat); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int sts_compute_M(Session& s, int n, cudaStream_t st) {
    const int N = s.N, R = s.R, R2 = R * R;
    sts_chain_kernel<<<1, 256, 0, st>>>(N, n, R, s.gram, s.chain); count_launch();
    EXAFAC_CHECK_LAUNCH();
    if (s.cfg.precision != EXAFAC_PREC_FP64) {
        // the mixed forms: Cholesky factors (the same row distribution)
        EXAFAC_TRY(launch_sts_factors_chol(N, n, R, 1e-8, s.chain, s.Emat, s.Phi, s.PhiP, s.eigV, s.eigL, s.vt, st));
    } else {
        EXAFAC_TRY(sts_eigen_factors(s, n, st));
    }
    EXAFAC_TRY(build_eigen_trees(s, n, st));
    if (s.cfg.precision != EXAFAC_PREC_FP64) {  // the mixed forms descend on FP32 copies
        EXAFAC_TRY(narrow_nodes(s.eigG, s.eigF, R, (int64_t)N * s.etree.node_count, st));
        EXAFAC_TRY(narrow_copy(s.Emat, s.EmatF, (int64_t)(N + 1) * R2, st));
        EXAFAC_TRY(narrow_nodes(s.PhiP, s.PhiPF, R, 1, st));
    }
    return EXAFAC_OK;
}

template <typename T>
struct StsModes {
    const T* treeG[kMaxModes];
    const T* U[kMaxModes];
    TreeShape rt[kMaxModes];
    int next[kMaxModes];
};

// STS_CP::KRPDrawSamples (sts_cp.hpp:203-300) at one rank, one sample per
// group of G warps: for each sampled mode k, an eigen-tree descent driven by h
// picks v and sets scaled_h = h * E[next(k)][v]; a row-tree descent driven by
// scaled_h picks the row and sets h *= U_k[row]
// (exact_leverage_tree.hpp:293-496 with no distributed levels).  Weight =
// R / (J h^T Phi h).  T = double: the reference's arithmetic on the FP64
// trees and factors; T = float (mixed forms): the same descents on FP32
// copies of the trees (summed in FP64, rounded once), factors, eigenvector
// rows and Phi.
template <typename T>
__global__ void sts_draw_kernel(int N, int n, int R, int G, int S, int64_t J, StsModes<T> m, TreeShape et,
                                const T* __restrict__ eigG, const T* __restrict__ E, const T* __restrict__ PhiP,
                                const double* __restrict__ uni, uint32_t* __restrict__ samples,
                                double* __restrict__ weights, DeviceStatus* status) {
    extern __shared__ __align__(16) unsigned char stsdyn[];
    const int P = node_stride<T>(R);  // node stride of the trees and of PhiP
    T *h, *sh, *q;
    int gi;
    const SampleGroup<T> grp = sample_group<T>(stsdyn, R, G, h, sh, q, gi);
    const int tg = grp.tg, nth = grp.nthreads();
    for (int64_t i = (int64_t)blockIdx.x * S + gi; i < J; i += (int64_t)gridDim.x * S) {
        for (int r = tg; r < R; r += nth) h[r] = T(1);
        bool empty = false;  // a descent ended in a leaf of zero mass: weight 0
        grp.sync();
        for (int k = 0; k < N; k++) {
            if (k == n) continue;
            // Eigen tree: descent by h, leaf v, scaled_h = h * E_next[v].
            const T* Ek = E + (int64_t)m.next[k] * R * R;
            grp.build_z(R, h);
            int64_t v = descend<T>(grp, et, R, eigG + (int64_t)k * et.node_count * P, Ek, h, q,
                                   (T)uni[((int64_t)k * 2 + 0) * J + i]);
            if (v >= R) {
                report(status, EXAFAC_ERR_DEVICE, 1, v, R);
                v = R - 1;
            }
            if (tg == 0) samples[i * N + n] = (uint32_t)v;
            for (int r = tg; r < R; r += nth) sh[r] = h[r] * Ek[v * R + r];
            grp.sync();
            // Row tree: descent by scaled_h, row, h *= U_k[row].
            grp.build_z(R, sh);
            int64_t row = descend<T>(grp, m.rt[k], R, m.treeG[k], m.U[k], sh, q,
                                     (T)uni[((int64_t)k * 2 + 1) * J + i], &empty);
            if (row >= m.rt[k].n) {
                report(status, EXAFAC_ERR_DEVICE, 2, row, m.rt[k].n);
                row = m.rt[k].n - 1;
            }
            if (tg == 0) samples[i * N + k] = (uint32_t)row;
            for (int r = tg; r < R; r += nth) h[r] *= m.U[k][row * R + r];
            grp.sync();
        }
        grp.build_z(R, h);
        const T hq = grp.quad(P, PhiP);
        // h^T Phi h > 0 for every sample the descents can reach in exact
        // arithmetic; a rounded zero or negative value (or an empty leaf)
        // gives the sample no weight instead of an infinite or NaN one.
        const bool ok = !empty && hq > T(0);
        if (tg == 0) weights[i] = ok ? (double)R / ((double)hq * (double)J) : 0.0;
        grp.sync();
    }
}

int sts_refresh_f32(Session& s, int k, cudaStream_t st) {
    if (s.cfg.sampler != EXAFAC_SAMPLER_STS_CP || s.cfg.precision == EXAFAC_PREC_FP64) return EXAFAC_OK;
    EXAFAC_TRY(narrow_copy(s.F.U[k], s.Uf[k], s.dims[k] * s.R, st));
    return narrow_nodes(s.treeG[k], s.treeF[k], s.R, s.rtree[k].node_count, st);
}

int sts_rebuild_tree(Session& s, int k, cudaStream_t st) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) return launch_tree_build(s.rtree[k], s.R, s.F.U[k], s.treeG[k], st);
    EXAFAC_TRY(narrow_copy(s.F.U[k], s.Uf[k], s.dims[k] * s.R, st));
    const uint32_t polls = s.wait_polls ? s.wait_polls : kSpinLimit;
    EXAFAC_TRY(launch_tree_build_f32(s.rtree[k], s.R, s.Uf[k], s.treeG[k], s.status, polls, st));
    return narrow_nodes(s.treeG[k], s.treeF[k], s.R, s.rtree[k].node_count, st);
}

template <typename T>
static int sts_draw_launch(Session& s, int n, int64_t J, const double* uni, const T* const* treeG, const T* const* U,
                           const T* eigG, const T* E, const T* PhiP, cudaStream_t st) {
    const int N = s.N;
    StsModes<T> m;
    for (int k = 0; k < kMaxModes; k++) {
        if (k < N) {
            m.treeG[k] = treeG[k];
            m.U[k] = U[k];
            m.rt[k] = s.rtree[k];
            int nx = k + 1;
            if (nx == n) nx++;
            if (nx > N) nx = N;
            m.next[k] = nx;
        } else {
            m.treeG[k] = nullptr;
            m.U[k] = nullptr;
            m.next[k] = 0;
        }
    }
    int G, S;
    sample_group_shape(s.R, sizeof(T), G, S);
    const size_t smem = (size_t)S * sample_group_bytes(s.R, sizeof(T));
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(sts_draw_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t blocks = std::max<int64_t>(std::min<int64_t>(ceil_div(J, S), 152 * 32), 1);
    sts_draw_kernel<T><<<(unsigned)blocks, S * G * 32, smem, st>>>(N, n, s.R, G, S, J, m, s.etree, eigG, E, PhiP, uni,
                                                                   s.samples, s.weights, s.status);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int sts_draw(Session& s, int n, int64_t J, const double* uni, cudaStream_t st) {
    if (s.cfg.precision == EXAFAC_PREC_FP64) {
        const double* treeG[kMaxModes];
        const double* U[kMaxModes];
        for (int k = 0; k < kMaxModes; k++) {
            treeG[k] = k < s.N ? s.treeG[k] : nullptr;
            U[k] = k < s.N ? s.F.U[k] : nullptr;
        }
        return sts_draw_launch<double>(s, n, J, uni, treeG, U, s.eigG, s.Emat, s.PhiP, st);
    }
    return sts_draw_bfs(s, n, J, uni, st);
}

}  // namespace exafac
