/*
 * exafac_gb300 — C ABI of the GB300 (sm_103a) sampled-ALS engine for sparse
 * CP decomposition (CP-ARLS-LEV and STS-CP samplers).
 *
 * Conventions
 *  - Every entry point returns an int status (EXAFAC_OK == 0); the text of the
 *    last failure on the calling thread is exafac_last_error().
 *  - Pointers named *_dev / device arrays are CUDA device pointers; `stream`
 *    is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - The library never allocates device memory: sessions run in a workspace
 *    the caller allocates after asking exafac_als_workspace_size().
 *  - Matrices are row-major float64 unless stated; factor matrix k is
 *    dims[k] x R.  Sample matrices are J x N uint32 (row j = one sampled
 *    Khatri-Rao row; column `mode` is scratch, as in the reference).
 *  - Calls enqueue work on `stream` and return without synchronising, except
 *    those documented as reading results back to the host.
 *
 * Each entry names the reference interface it replaces
 * (vbharadwaj-bk/rdist_tensor, exafac/cpp_ext/...).
 */
#ifndef EXAFAC_GB300_H
#define EXAFAC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EXAFAC_ABI_VERSION 1
#define EXAFAC_MAX_MODES 8
#define EXAFAC_MAX_RANK 128

enum {
    EXAFAC_OK = 0,
    EXAFAC_ERR_ARG = 1,         /* invalid argument (checked on the host)            */
    EXAFAC_ERR_CUDA = 2,        /* a CUDA runtime call failed                        */
    EXAFAC_ERR_DEVICE = 3,      /* a kernel found an out-of-range index (see below)  */
    EXAFAC_ERR_TIMEOUT = 4,     /* a bounded device-side wait ran out                */
    EXAFAC_ERR_UNSUPPORTED = 5, /* shape or option outside what the build supports   */
    EXAFAC_ERR_WORKSPACE = 6    /* workspace smaller than exafac_als_workspace_size  */
};

enum { EXAFAC_SAMPLER_CP_ARLS_LEV = 0, EXAFAC_SAMPLER_STS_CP = 1 };

/* Arithmetic of the sampled-design products (design Gram, solve, leverage
 * scores).  FP64 follows the reference.  The mixed forms compute them in
 * TF32 or BF16 with FP32 accumulation and keep FP64 for the Gram Hadamard
 * chain, the R x R solve (plus one refinement step) and the tree sums. */
enum { EXAFAC_PREC_FP64 = 0, EXAFAC_PREC_TF32 = 1, EXAFAC_PREC_BF16 = 2 };

/* Value preprocessing of SparseTensor (sparse_tensor.hpp:44-63). */
enum { EXAFAC_PRE_NONE = 0, EXAFAC_PRE_LOG_COUNT = 1, EXAFAC_PRE_ONES = 2 };

const char* exafac_last_error(void);
int exafac_abi_version(void);

/* Number of kernels this library has launched since it was loaded. */
long long exafac_kernel_launches(void);

/* ---------------------------------------------------------------------------
 * Single routines (stateless).  They exist so each reference routine can be
 * checked on its own; the session API below chains them.
 * ------------------------------------------------------------------------- */

/* PartitionTree node count for n rows in leaves of F rows
 * (partition_tree.hpp:82-102). */
int64_t exafac_tree_node_count(int64_t n, int32_t F);

/* PartitionTree::build_tree (partition_tree.hpp:117-167): G[node] = U_blk^T U_blk
 * for leaves, pairwise sums above.  G is node_count x R x R. */
int exafac_tree_build(int64_t n, int32_t F, int32_t R, const double* U_dev, double* G_dev, void* stream);

/* The mixed forms' PartitionTree::build_tree from an FP32 copy of U (n x R,
 * device): leaf Grams on the tensor cores (TF32 hi + lo parts, 32 <= R,
 * F <= 128) or as compensated FP32 sums, internal sums in FP64; G as for
 * exafac_tree_build. */
int exafac_tree_build_f32(int64_t n, int32_t F, int32_t R, const float* U_dev, double* G_dev, void* stream);

/* PartitionTree::PTSample (partition_tree.hpp:204-380): for each of J samples
 * descend by the quadratic forms x_j^T G x_j with the explicit uniform
 * draws_dev[j]; write the chosen row to rows_out_dev[j * rows_stride] and
 * multiply hmul_dev row j by U[row]. */
int exafac_tree_sample(int64_t n, int32_t F, int32_t R, const double* G_dev, const double* U_dev, int64_t J,
                       const double* x_dev, double* hmul_dev, const double* draws_dev, uint32_t* rows_out_dev,
                       int64_t rows_stride, void* stream);

/* The quadratic forms of the mixed forms' breadth-first STS-CP descents
 * (the per-level node masses of PartitionTree::PTSample,
 * partition_tree.hpp:204-380, in FP32): q[j] = x_j^T G_{node[j]} x_j for J
 * FP32 vectors (J x R, device) and node indices into G, packed upper
 * triangles (rows in order, node stride R (R + 1) / 2 rounded up to a
 * multiple of 4 floats).  use_tc = 1 (R >= 32): on the tensor cores
 * (tcgen05); 2: the same arithmetic with the node's operand kept resident
 * across tiles (the kernel of the root and shallow descent levels, for long
 * runs of equal node; results equal to use_tc = 1 bit for bit); 0: FP32 on
 * the CUDA cores.  Slots of equal node next to each other share one staging
 * of the node. */
int exafac_quad_forms_f32(int32_t R, int64_t J, const float* X_dev, const int64_t* node_dev, const float* G_dev,
                          float* q_dev, int32_t use_tc, void* stream);

/* LAPACKE_dsyev('V','U') as used by the reference (sts_cp.hpp:110-116):
 * eigenvalues ascending in lambda_dev[R], eigenvector v in column v of V_dev
 * (V[u * R + v]).  Reads the upper triangle of A_dev.  One-CTA Jacobi. */
int exafac_syev(int32_t R, const double* A_dev, double* V_dev, double* lambda_dev, void* workspace_dev,
                size_t workspace_bytes, void* stream);

/* compute_pinv_square (common.h:405-443): symmetric pseudo-inverse dropping
 * eigenvalues <= tol (the reference uses 1e-11).  out_dev is full symmetric. */
int exafac_pinv_square(int32_t R, const double* A_dev, double* out_dev, double tol, void* workspace_dev,
                       size_t workspace_bytes, void* stream);

/* Device workspace bytes exafac_syev / exafac_pinv_square need for rank R. */
size_t exafac_dense_workspace_bytes(int32_t R);

/* exafac_pinv_square without a workspace argument, for callers that cannot
 * allocate device memory (their memory belongs to another framework's pool,
 * or allocation is not allowed where they run).  No counterpart in the
 * reference.  Scratch is a static 128 KiB device array shared by all calls
 * on a device: R must be <= 128; calls that overlap on the GPU race on it.
 * The first call on each device looks up the array's address
 * (cudaGetSymbolAddress), so make it before any stream capture.  The address
 * is kept for the life of the process: after a device reset
 * (cudaDeviceReset, or a reset of the primary context) the module is loaded
 * again and the kept address is stale, so do not call this entry point on a
 * device that has been reset since its first call. */
int exafac_pinv_square_static(int32_t R, const double* A_dev, double* out_dev, double tol, void* stream);

/* ---------------------------------------------------------------------------
 * Session: SparseTensor + LowRankTensor + Sampler + AccumulatorStationary
 * (py_module.cpp:37-77) on one GPU.
 * ------------------------------------------------------------------------- */
typedef struct exafac_als_s* exafac_als_t;

typedef struct {
    int32_t N;                       /* modes (2..8)                          */
    int32_t R;                       /* target rank (1..128)                  */
    int64_t dims[EXAFAC_MAX_MODES];  /* mode sizes                            */
    int64_t nnz;                     /* nonzeros                              */
    int64_t J_max;                   /* largest sample count per step         */
    int32_t sampler;                 /* EXAFAC_SAMPLER_*                      */
    int32_t precision;               /* EXAFAC_PREC_*                         */
    int32_t preprocessing;           /* EXAFAC_PRE_*                          */
    int32_t reserved;
} exafac_als_config;

/* LowRankTensor (low_rank_tensor.hpp:10-54): caller-owned device buffers. */
typedef struct {
    double* U[EXAFAC_MAX_MODES]; /* dims[k] x R, row-major */
    double* sigma;               /* R                      */
} exafac_factors;

/* Counters of the last step, read back by exafac_als_step_info. */
typedef struct {
    int64_t unique_samples; /* J_u after deduplication                      */
    int64_t hits;           /* nonzeros found (nonzeros_iterated, per step)  */
    int64_t touched_rows;   /* rows of the updated factor that are nonzero  */
    int64_t hits_total;     /* sum of `hits` over all steps since creation  */
    int32_t device_status;  /* EXAFAC_OK or the first device-side error     */
    int32_t pad;
} exafac_step_info;

/* Bytes of device workspace: `persistent` lives as long as the session
 * (sorted per-mode copies, fiber hash tables, sampler state, step scratch);
 * `setup` is only needed during exafac_als_init. */
int exafac_als_workspace_size(const exafac_als_config* cfg, size_t* persistent_bytes, size_t* setup_bytes);

/* Creates a session over a caller-allocated persistent workspace (256-byte
 * aligned device memory of at least persistent_bytes). */
int exafac_als_create(const exafac_als_config* cfg, void* persistent_dev, size_t persistent_bytes, exafac_als_t* out);
int exafac_als_destroy(exafac_als_t s);

/* SparseTensor ctor preprocessing + AccumulatorStationary::
 * initialize_ground_truth_for_als (accumulator_stationary.hpp:38-137) +
 * sampler construction (cp_arls_lev.hpp:14-23 / sts_cp.hpp:32-57).
 * idx_dev: nnz x N uint32 coordinates (< dims), vals_dev: nnz float64 (copied
 * into the workspace, then preprocessed).  The session keeps `factors` (the
 * caller keeps the buffers alive).  Writes ||X|| (after preprocessing) to
 * *tensor_norm (host; this call synchronises). */
int exafac_als_init(exafac_als_t s, const uint32_t* idx_dev, const double* vals_dev, const exafac_factors* factors,
                    void* setup_dev, size_t setup_bytes, double* tensor_norm, void* stream);

/* Sampler::KRPDrawSamples (sampler.hpp:23-27) for `mode`.  Uniforms:
 * CP-ARLS-LEV [N][J] (row `mode` unused), STS-CP [N][2][J] (eigen-tree then
 * row-tree draws per sampled mode).  perms_dev (CP-ARLS-LEV only, may be
 * NULL = identity): [N][J], sample j of mode k takes draw perms[k][j]
 * (cp_arls_lev.hpp:61-66).  uniforms_dev NULL: the session's own Philox
 * stream supplies them.  Writes J x N samples and J weights. */
int exafac_als_draw(exafac_als_t s, int32_t mode, int64_t J, const double* uniforms_dev, const uint32_t* perms_dev,
                    uint32_t* samples_dev, double* weights_dev, void* stream);

/* AccumulatorStationary::execute_ALS_step (accumulator_stationary.hpp:139-295):
 * draw, deduplicate, design rows + Gram + pinv, sampled MTTKRP, U_mode =
 * MTTKRP * pinv, column renormalisation into sigma, sampler update. */
int exafac_als_step(exafac_als_t s, int32_t mode, int64_t J, const double* uniforms_dev, const uint32_t* perms_dev,
                    void* stream);

/* SortIdxLookup::csr_based_spmm (sort_lookup.hpp:238-375) on the mode's
 * sorted copy: for Ju deduplicated samples (Ju x N, device) and design rows
 * (Ju x R, device), out (dims[mode] x R, device) = sum over the nonzeros whose
 * coordinates off `mode` equal a sample's of value * design row, accumulated
 * into the nonzero's mode-`mode` row.  Uses the session's step scratch;
 * synchronises.  The hit count is readable through exafac_als_step_info. */
int exafac_als_sampled_mttkrp(exafac_als_t s, int32_t mode, int64_t Ju, const uint32_t* samples_dev,
                              const double* design_dev, double* out_dev, void* stream);

/* ExactALS::execute_ALS_step (exact_als.hpp:90-143): exact MTTKRP over all
 * nonzeros; used for the "-p exact" preprocessing (decompose.py:82-96).  The
 * sampler state is refreshed for `mode`. */
int exafac_als_exact_step(exafac_als_t s, int32_t mode, void* stream);

/* ALS_Optimizer::compute_exact_fit -> SparseTensor::compute_exact_fit
 * (sparse_tensor.hpp:288-356).  Synchronises; *fit is a host double. */
int exafac_als_fit(exafac_als_t s, double* fit, void* stream);

/* Fit estimate with zero sampling (the reference's legacy
 * DistLowRank.compute_estimated_fit, exafac/low_rank_tensor.py:110-184):
 * 1 - sqrt(sum over nonzeros of (x - m)^2 + (prod dims - nnz) * mean of m^2
 * over the zero samples kept) / ||X||, m the model value.  Z coordinates are
 * drawn uniformly over the index space (zero_idx_dev, Z x N uint32, or NULL
 * for Philox4x32-10 keyed by seed); those that are nonzeros of the tensor are
 * dropped, found exactly through the session's mode-0 fibre hash table (the
 * reference used a Bloom filter, bloom_filter.cpp:198-252).  The reference
 * takes Z = (1 / alpha - 1) nnz with alpha = 0.5.  Writes *fit and the number
 * of zero samples kept (*kept, may be NULL); synchronises. */
int exafac_als_estimated_fit(exafac_als_t s, int64_t Z, const uint32_t* zero_idx_dev, uint64_t seed, double* fit,
                             int64_t* kept, void* stream);

/* Seeds the session's Philox stream used when uniforms_dev is NULL. */
int exafac_als_set_seed(exafac_als_t s, uint64_t seed);

/* Region timers of ALS_Optimizer (als_optimizer.hpp:19-27).  When enabled,
 * each exafac_als_step records CUDA events at its region borders on its
 * stream and returns without waiting for them; exafac_als_region_times waits
 * for the steps recorded so far and returns the seconds accumulated since
 * enabling, in the order leverage_sampling, row_gather, design_matrix_prep,
 * spmm, dense_reduce, postprocessing, sampler_update.  At most 512 steps stay
 * pending; a later step first waits for the oldest. */
int exafac_als_enable_timing(exafac_als_t s, int32_t enable);
int exafac_als_region_times(exafac_als_t s, double* out7);

/* `count` sweeps (steps 0..N-1 each; round loop of als_optimizer.hpp:40-124
 * without its timers) at J samples per step.  uniforms_dev: null for the
 * session's Philox stream, or N per-step blocks laid out as for
 * exafac_als_step, read again on every sweep.  After any factor has had a
 * sampled update, one sweep is captured into a CUDA graph on an internal
 * stream and replayed (the capture is kept for the same J and uniforms
 * pointer, and dropped by exafac_als_init / exafac_als_set_seed); results are
 * those of calling exafac_als_step N x count times.  Region timing must be off. */
int exafac_als_sweeps(exafac_als_t s, int64_t J, int32_t count, const double* uniforms_dev, void* stream);

/* Failure-detection test hook (no counterpart in the reference, which has no
 * device-side waits).  The row sort of each step waits, per tile, for the
 * status words of earlier tiles (a decoupled look-back); a wait gives up after
 * `polls` polls (0 = the default, 2^22, about half a second) and the step then
 * reports EXAFAC_ERR_TIMEOUT through exafac_als_step_info.device_status, with
 * no hits processed.  withhold_tile >= 0 makes that tile of the first digit
 * pass publish no status, so the waits on it run out; -1 turns this off. */
int exafac_als_set_wait_limit(exafac_als_t s, uint32_t polls, int64_t withhold_tile);

/* Copies the last step's counters to the host (synchronises). */
int exafac_als_step_info(exafac_als_t s, exafac_step_info* out, void* stream);

/* Device views of the last step's intermediates (for tests): deduplicated
 * samples [J_u x N], their weights [J_u], the design Gram and its pinv
 * [R x R].  Pointers stay valid until the next step. */
int exafac_als_last_dedup(exafac_als_t s, const uint32_t** samples_dev, const double** weights_dev,
                          const double** design_gram_dev, const double** design_pinv_dev);

/* ---------------------------------------------------------------------------
 * Generalized CP on sampled entries.  No counterpart in the reference: these
 * are the forward and adjoint of a sampled-MTTKRP torch.autograd.Function
 * (rdist_tensor_gb300/gcp.py) for gradient-based CP with Poisson or
 * Bernoulli losses.  Nearest reference relatives: execute_exact_mttkrp
 * (sort_lookup.hpp:440-495) and the zero-sampling fit estimate
 * (exafac/low_rank_tensor.py:110-184).
 *
 * Factors are device row-major dims[k] x R matrices of `dtype`; idx is a
 * device int32 [J x N] coordinate array.  Entries with a coordinate outside
 * dims are skipped (model value 0, no gradient) and set *status_dev to 1
 * when status_dev is not null.
 * ------------------------------------------------------------------------- */
enum { EXAFAC_DTYPE_F32 = 0, EXAFAC_DTYPE_F64 = 1 };

/* m[j] = sum_r prod_k U_k[idx[j,k], r]. */
int exafac_cp_sampled_model(int32_t N, int32_t R, const int64_t* dims_host, int64_t J, const int32_t* idx_dev,
                            const void* const* factors_dev, void* m_dev, int32_t dtype, int32_t* status_dev,
                            void* stream);

/* Adjoint of the model: grads[n][idx[j,n], :] += grad_m[j] * prod_{k != n}
 * U_k[idx[j,k], :] for every n with grads[n] != null (accumulates; the
 * Khatri-Rao rows are recomputed, not stored; atomic accumulation). */
int exafac_cp_sampled_adjoint(int32_t N, int32_t R, const int64_t* dims_host, int64_t J, const int32_t* idx_dev,
                              const void* grad_m_dev, const void* const* factors_dev, void* const* grads_dev,
                              int32_t dtype, int32_t* status_dev, void* stream);

/* Stratified entry sample: J_nz nonzeros drawn uniformly with replacement
 * (value x, weight nnz / J_nz) followed by J_z uniform coordinates taken as
 * zeros (value 0, weight (prod dims - nnz) / J_z); Philox4x32-10 keyed by
 * seed at counter `counter`.  Outputs idx [J x N], x [J], w [J]. */
int exafac_gcp_sample_entries(int32_t N, const int64_t* dims_host, int64_t nnz, const int32_t* nz_idx_dev,
                              const void* nz_vals_dev, int64_t J_nz, int64_t J_z, uint64_t seed, uint64_t counter,
                              int32_t* idx_dev, void* x_dev, void* w_dev, int32_t dtype, void* stream);

/* One Adam step over `count` (<= 8) device tensors of `dtype` in one launch,
 * fused with the projection onto x >= lower when project != 0: per element
 *   m = m + (1 - beta1) (g - m);  v = beta2 v + (1 - beta2) g^2;
 *   p = p - lr / (1 - beta1^step) * m / (sqrt(v) / sqrt(1 - beta2^step) + eps);
 *   p = max(p, lower)   (projection; a NaN stays NaN)
 * in the tensors' own precision: the update of torch.optim.Adam (no weight
 * decay, no amsgrad), the optimizer of gradient-based GCP, followed by the
 * nonnegativity projection of its Poisson and Bernoulli losses.  `step` is
 * the step count after this update (>= 1).  grads (or one entry of it) may be
 * null: a zero gradient.  No reference counterpart (the reference has no
 * GCP). */
int exafac_adam_step(int32_t count, void* const* params_dev, const void* const* grads_dev, void* const* exp_avg_dev,
                     void* const* exp_avg_sq_dev, const int64_t* numel_host, int32_t dtype, double lr, double beta1,
                     double beta2, double eps, int64_t step, int32_t project, double lower, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EXAFAC_GB300_H */
