// Sampled-ALS session state and the kernels of one step.
//
// Data layout in HBM (all inside the caller's workspace):
//   idx      nnz x N uint32    coordinates as given (fit, exact MTTKRP)
//   vals     nnz float64       preprocessed values
//   per mode n (SortIdxLookup, sort_lookup.hpp:37-102):
//     rows_n  nnz uint32       mode-n coordinate, nonzeros ordered by the
//                              packed key of the other coordinates
//     vals_n  nnz float64      values in the same order
//     slots_n hash table       fiber key -> [start, start + len) in rows_n
//   sampler state per mode (scores + CDF for CP-ARLS-LEV; packed Gram tree +
//   Gram for STS-CP), step scratch sized for J_max samples and nnz hits.
#pragma once
#include "common.cuh"
#include "tree.cuh"

namespace exafac {

constexpr uint32_t kEmpty = 0xffffffffu;
// CDFs up to this length are summed strictly in order (bit compatible with
// libstdc++).  The two serial FP64 chains cost ~64 cycles per element on GB300
// (a dependent FP64 add), so longer CDFs take the blockwise scan.
constexpr int64_t kExactCdfMax = 512;
constexpr int kGuideBuckets = 1 << 16;   // buckets of the CDF guide tables (a power of two)
constexpr int kExpandChunk = 256;  // hits per warp chunk in the hit expansion
constexpr int kSortEpochSlot = 14;  // counters[] slot of the row sort's look-back epoch
constexpr int kRngSlot = 15;              // counters[] slot of the session's Philox counter

struct Slot1 {
    unsigned long long key;
    unsigned int start, len;
};
struct Slot2 {
    unsigned long long lo, hi;
    unsigned int start, len;
    unsigned long long pad;
};

struct Lookup {
    uint32_t* rows = nullptr;
    double* vals = nullptr;
    void* slots = nullptr;  // Slot1[nslots] or Slot2[nslots]
    int64_t nslots = 0;     // power of two
    int kw = 1;             // key words
    KeySpec spec;
};

struct FactorPtrs {  // factor matrices passed by value to kernels
    const double* U[kMaxModes];
};

// Sample state of the breadth-first STS-CP draws of the mixed forms
// (bfs_sampler.cu), J_max entries each unless stated.
struct BfsState {
    float* h = nullptr;       // J x R: product of the chosen rows
    float* sh = nullptr;      // J x R: h scaled by the chosen eigenvector row
    float* m = nullptr;       // root mass of the current descent (then h^T Phi h)
    float2* lh = nullptr;     // (low, high) of the current descent
    int64_t* node = nullptr;  // current node
    int32_t* order[2] = {nullptr, nullptr};  // slot -> sample, ordered by node (ping-pong)
    int cur = 0;
    uint32_t* flag = nullptr;  // by slot: went left (or stayed at a leaf)
    int64_t* SL = nullptr;     // J + 1: exclusive scan of flag
    int64_t* off[2] = {nullptr, nullptr};  // slot ranges of a level's nodes (ping-pong)
    int32_t* v = nullptr;      // eigen-tree leaf of each sample
    int32_t* empty = nullptr;  // a descent ended in a leaf of zero mass
};

struct Session {
    exafac_als_config cfg;
    int N = 0, R = 0, P = 0;
    int64_t dims[kMaxModes] = {0};
    int64_t nnz = 0, Jmax = 0, Imax = 0;
    Arena arena;
    bool initialized = false;
    double tensor_norm = 0.0;
    exafac_factors F;

    uint32_t* idx = nullptr;
    double* vals = nullptr;
    Lookup look[kMaxModes];

    // CP-ARLS-LEV state
    double* scores[kMaxModes] = {nullptr};
    double* scores_c = nullptr;  // Imax: the step's leverage scores by touched-row index (compact, for the CDF)
    double* cdf[kMaxModes] = {nullptr};
    uint32_t* guide[kMaxModes] = {nullptr};
    bool cdf_compact[kMaxModes] = {false};  // CDF over nzrows[k] (a sampled update) rather than all rows  // kGuideBuckets + 1: guide[b] = lower_bound(cdf, b / kGuideBuckets)
    double* cdf_total = nullptr;  // [N] sum of the scores (log-weight numerator)
    // STS-CP state
    TreeShape rtree[kMaxModes];
    double* treeG[kMaxModes] = {nullptr};
    TreeShape etree;
    double* eigG = nullptr;    // [N] eigen trees, etree.node_count * P each
    double* gram = nullptr;    // [N] R x R factor Grams (full)
    double* chain = nullptr;   // [N] R x R suffix Hadamard products
    double* Emat = nullptr;    // [N+1] R x R scaled eigenvector rows
    double* eigV = nullptr;    // [N+1] R x R eigenvectors
    double* eigL = nullptr;    // [N+1] R eigenvalues
    double* Phi = nullptr;     // R x R (full)
    double* PhiP = nullptr;    // packed
    double* vt = nullptr;      // Jacobi scratch, N+1 matrices
    // FP32 copies the mixed forms' STS-CP descents read (rounded from the FP64
    // arrays after every change): row trees, factors, eigen trees, E, Phi
    float* treeF[kMaxModes] = {nullptr};
    float* Uf[kMaxModes] = {nullptr};
    float* eigF = nullptr;
    float* EmatF = nullptr;
    float* PhiPF = nullptr;
    BfsState bfs;

    // nonzero-row tracking per factor (rows outside the list are zero)
    bool dense[kMaxModes] = {false};
    uint32_t* nzrows[kMaxModes] = {nullptr};
    int64_t* nzcount = nullptr;  // [N]

    // step scratch
    double* uni = nullptr;  // N x 2 x Jmax
    uint32_t* samples = nullptr;
    double* weights = nullptr;
    int64_t dtab = 0;  // dedup table size (power of two)
    int32_t* d_owner = nullptr;
    int32_t* d_minj = nullptr;
    int32_t* d_count = nullptr;
    int32_t* slot_of = nullptr;
    Key128* dkey = nullptr;         // J: packed dedup key of each sample
    uint32_t* flags = nullptr;  // J: per-tile representative counts of the deduplication
    uint32_t* sd = nullptr;
    double* wd = nullptr;
    int64_t* counters = nullptr;  // [0] J_u, [1] H, [2] touched, [3..] scratch, [kRngSlot] Philox counter
    double* D = nullptr;          // Jmax x R design rows (scaled twice)
    double* part = nullptr;       // Gram partials
    int64_t part_rows = 0;
    double* dgram = nullptr;      // R x R design Gram
    double* dpinv = nullptr;      // R x R its pseudo-inverse
    uint32_t* f_start = nullptr;
    uint32_t* f_len = nullptr;
    int64_t* f_off = nullptr;
    uint32_t* touched = nullptr;  // Imax: rows with hits, increasing
    int64_t* seg_start = nullptr; // Imax + 1: first sorted hit of each touched row, then H
    double* ugram = nullptr;      // R x R
    double* ngram = nullptr;      // R x R normalised factor Gram
    double* upinv = nullptr;      // R x R
    double* fitpart = nullptr;
    DeviceStatus* status = nullptr;
    void* scan_sc = nullptr;
    int64_t* dims_dev = nullptr;  // [kMaxModes]
    double* Mexact = nullptr;     // Imax x R (exact MTTKRP)
    double* scal = nullptr;       // [8] device scalars (norms, fit terms)
    // hits: sample order (ex_*), then sorted by row (hitsort.cu)
    uint32_t* ex_j = nullptr;         // nnz: sample of hit h
    double* ex_val = nullptr;         // nnz: value of hit h
    uint32_t* hit_key[2] = {nullptr, nullptr};  // nnz each: output rows (sort ping-pong)
    uint32_t* hit_pay[2] = {nullptr, nullptr};  // nnz each: hit indices (sort ping-pong)
    const uint32_t* key_sorted = nullptr;       // the sorted rows of the current step
    const uint32_t* pay_sorted = nullptr;       // their hit indices (FP64 form)
    uint64_t* pay64[2] = {nullptr, nullptr};    // nnz each, mixed forms: packed (sample, FP32 value) (ping-pong)
    const uint64_t* pay64_sorted = nullptr;     // the sorted packed hits (mixed forms)
    uint64_t* os_status = nullptr;    // tile stride x 256: look-back status words of the row sort
    uint32_t* os_aux = nullptr;       // row sort: 4 tile counters, 4 x 256 digit histograms; run pass: 1 tile counter
    double* Mc = nullptr;             // Imax x R: MTTKRP rows, indexed by row
    double* carry_first = nullptr;  // chunks x kCarryStride
    double* carry_last = nullptr;   // chunks x kCarryStride
    uint32_t* carry_row = nullptr;  // chunks: row continuing past the chunk, or 0xffffffff
    uint32_t* carry_seg = nullptr;  // chunks: that row's touched-row index (compact Mc)
    uint32_t* chunk_seg = nullptr;  // chunks of kSegChunkF32 sorted hits: run index of the first hit
    uint32_t* expand_first = nullptr;  // ceil(nnz / kExpandChunk) + 1: sample owning each expansion chunk's first hit
    float* Uc = nullptr;            // Imax x f32_row_stride(R), mixed forms: solved rows by touched-row index
    uint32_t* rowbits = nullptr;    // ceil(Imax / 32): rows touched by the current step
    float* Df = nullptr;          // Jmax x f32_row_stride(R) design rows (mixed forms)

    uint64_t seed = 0x5eed;  // Philox key; the stream counter is counters[kRngSlot] on the device
    // Look-back waits of the row sort: poll limit, and (test hook, -1 = off)
    // a tile of the first digit pass that publishes no status.
    uint32_t wait_polls = kSpinLimit;
    int64_t withhold_tile = -1;
};

// ---- sampler kernels (sampler_kernels.cu)
int gen_uniforms(Session& s, double* out, int64_t count, cudaStream_t st);
int arls_build_cdf(Session& s, int k, const uint32_t* list, const int64_t* count_dev, cudaStream_t st);
int arls_leverage(Session& s, int k, bool all_rows, const double* pinv, cudaStream_t st);
int arls_draw(Session& s, int n, int64_t J, const double* uni, const uint32_t* perms, cudaStream_t st);
int sts_compute_M(Session& s, int n, cudaStream_t st);
int sts_draw(Session& s, int n, int64_t J, const double* uni, cudaStream_t st);
// The mixed forms' STS-CP draws, breadth first (bfs_sampler.cu).
int sts_draw_bfs(Session& s, int n, int64_t J, const double* uni, cudaStream_t st);
// Tensor-core descents (bfs_sampler.cu): used for R >= kTcMinRank.
constexpr int kTcMinRank = 32;
// FP32 copies of factor k and its row tree (mixed STS-CP sessions; else a no-op).
int sts_refresh_f32(Session& s, int k, cudaStream_t st);
// Row tree of mode k after a sampled update: FP64 build (FP64 form), or the
// FP32-copy build with FP64 internal sums and the FP32 copies (mixed forms).
int sts_rebuild_tree(Session& s, int k, cudaStream_t st);

// ---- step kernels (step_kernels.cu)
int dedup(Session& s, int n, int64_t J, cudaStream_t st);
int design_gram(Session& s, int n, int64_t J, cudaStream_t st);
int design_pinv(Session& s, cudaStream_t st);
int gram_rows(Session& s, const double* A, int64_t rows, const uint32_t* rowlist, const int64_t* count_dev,
              double* out_full, cudaStream_t st);
int lookup_hits(Session& s, int n, int64_t J, bool packed, cudaStream_t st);
int keep_touched(Session& s, int n, cudaStream_t st);
int lookup_fibers(Session& s, int n, int64_t J, cudaStream_t st);
int gram_reduce_to(Session& s, int64_t nblk, double* out, cudaStream_t st);
int sigma_and_gram(Session& s, cudaStream_t st);
int scale_rows_if_degenerate(Session& s, int n, cudaStream_t st);

// ---- load-balanced MTTKRP and post-processing, R <= 32 (post_kernels.cu)
constexpr int kSegChunkHits = 128;  // hits per chunk of the FP64 segmented reduction
constexpr int kSegChunkF32 = 64;    // hits per chunk of the FP32 segmented reduction (a multiple of 32)
// FP32 row stride of the design rows (Df) and MTTKRP rows (Mc): R rounded up
// to a multiple of 4, so a row is a whole number of float4s.
__host__ __device__ inline int f32_row_stride(int R) { return (R + 3) & ~3; }
constexpr int kCarryStride = 32;  // carry rows padded to 32 columns (R <= 32)

// ---- hits grouped by output row (hitsort.cu)
size_t hitsort_tile_stride(int64_t nnz);
// packed: carry (sample, FP32 value) through the sort (mixed forms) instead of
// the hit index.
int hits_by_row(Session& s, int n, bool packed, cudaStream_t st);
// All nonzeros sorted by their mode-n index (key_sorted, pay_sorted = position).
int nonzeros_by_row(Session& s, int n, cudaStream_t st);
int mttkrp_solve_balanced(Session& s, int n, cudaStream_t st);
int normalize_balanced(Session& s, int n, bool arls, cudaStream_t st);
int mttkrp_scatter_out(Session& s, double* out, cudaStream_t st);
// 32 < R <= 128 (wide_kernels.cu): MTTKRP + solve + Gram, and renormalisation,
// in FP64 (FP64 form) or FP32 (mixed forms).
// before_solve (may be null): an event the solve waits for (the pseudo-inverse).
int mttkrp_solve_wide(Session& s, int n, cudaStream_t st, cudaEvent_t before_solve = nullptr);
int normalize_wide(Session& s, int n, bool arls, cudaStream_t st);
int spmm_solve(Session& s, int n, cudaStream_t st);
int spmm_solve_into(Session& s, int n, const double* Phi, double* out, cudaStream_t st);
int normalize_factor(Session& s, int n, bool all_rows, cudaStream_t st);
int clear_dense_factor(Session& s, int n, cudaStream_t st);
int zero_old_rows(Session& s, int n, cudaStream_t st);
int fit_residual(Session& s, double* out_dev, cudaStream_t st);
// Zero-sampling fit estimate (estfit.cu); synchronises.
int estimated_fit(Session& s, int64_t Z, const uint32_t* zero_idx, uint64_t seed, double* fit, int64_t* kept,
                  cudaStream_t st);
int exact_mttkrp(Session& s, int n, double* M, cudaStream_t st);
int matmul_rows_sym(Session& s, const double* M, const double* Phi, double* U, int64_t rows, cudaStream_t st);
int chain_gram(Session& s, int skip, double* out, cudaStream_t st);

// ---- setup kernels (setup_kernels.cu)
size_t setup_bytes(const Session& s);
int build_lookup(Session& s, int n, void* setup, size_t setup_bytes, cudaStream_t st);
int preprocess_values(Session& s, const double* vals_in, cudaStream_t st);

}  // namespace exafac
