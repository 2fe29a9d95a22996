// Host orchestration of the sampled-ALS session and its C ABI.
//
// One step (AccumulatorStationary::execute_ALS_step, accumulator_stationary.hpp:
// 139-295, at one rank) is ~30 launches on the caller's stream with no host
// synchronisation: data-dependent sizes (unique samples, hits, touched rows)
// stay on the device and kernels read them from there, so a sweep can be
// captured in a CUDA graph.
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

#include "dense.cuh"
#include "engine.cuh"
#include "prims.cuh"

namespace exafac {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static int64_t next_pow2(int64_t x) {
    int64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Carves the persistent workspace.  With arena.base == nullptr it only sizes.
static void carve(Session& s) {
    Arena& a = s.arena;
    const int N = s.N, R = s.R, R2 = R * R, P = s.P;
    const int64_t nnz = s.nnz, J = s.Jmax, I = s.Imax;
    s.idx = a.take<uint32_t>(nnz * N);
    s.vals = a.take<double>(nnz);
    for (int n = 0; n < N; n++) {
        Lookup& L = s.look[n];
        L.rows = a.take<uint32_t>(nnz);
        L.vals = a.take<double>(nnz);
        L.slots = L.kw == 1 ? (void*)a.take<Slot1>(L.nslots) : (void*)a.take<Slot2>(L.nslots);
    }
    if (s.cfg.sampler == EXAFAC_SAMPLER_CP_ARLS_LEV) {
        for (int k = 0; k < N; k++) {
            s.scores[k] = a.take<double>(s.dims[k]);
            s.cdf[k] = a.take<double>(s.dims[k]);
            s.guide[k] = a.take<uint32_t>(kGuideBuckets + 1);
        }
        int64_t imax = 1;
        for (int k = 0; k < N; k++) imax = std::max<int64_t>(imax, s.dims[k]);
        s.scores_c = a.take<double>(imax);
    } else {
        for (int k = 0; k < N; k++) s.treeG[k] = a.take<double>(s.rtree[k].node_count * P);
        s.eigG = a.take<double>((int64_t)N * s.etree.node_count * P);
        if (s.cfg.precision != EXAFAC_PREC_FP64) {
            const int Pf = packed_stride_f32(R);
            for (int k = 0; k < N; k++) {
                s.treeF[k] = a.take<float>(s.rtree[k].node_count * Pf);
                s.Uf[k] = a.take<float>(s.dims[k] * R);
            }
            s.eigF = a.take<float>((int64_t)N * s.etree.node_count * Pf);
            s.EmatF = a.take<float>((int64_t)(N + 1) * R2);
            s.PhiPF = a.take<float>(Pf);
            BfsState& b = s.bfs;
            b.h = a.take<float>(J * R);
            b.sh = a.take<float>(J * R);
            b.m = a.take<float>(J);
            b.lh = a.take<float2>(J);
            b.node = a.take<int64_t>(J);
            b.order[0] = a.take<int32_t>(J);
            b.order[1] = a.take<int32_t>(J);
            b.flag = a.take<uint32_t>(J);
            b.SL = a.take<int64_t>(J + 1);
            int64_t widest = std::max<int64_t>(s.etree.leaf_count, 1);  // nodes of the widest level
            for (int k = 0; k < N; k++) widest = std::max<int64_t>(widest, s.rtree[k].leaf_count);
            b.off[0] = a.take<int64_t>(2 * widest + 2);
            b.off[1] = a.take<int64_t>(2 * widest + 2);
            b.v = a.take<int32_t>(J);
            b.empty = a.take<int32_t>(J);
        }
    }
    s.cdf_total = a.take<double>(N);
    s.gram = a.take<double>((int64_t)N * R2);
    s.chain = a.take<double>((int64_t)N * R2);
    s.Emat = a.take<double>((int64_t)(N + 1) * R2);
    s.eigV = a.take<double>((int64_t)(N + 1) * R2);
    s.eigL = a.take<double>((int64_t)(N + 1) * R);
    s.Phi = a.take<double>(R2);
    s.PhiP = a.take<double>(P);
    s.vt = a.take<double>((int64_t)syev_scratch_doubles(R, N + 1));
    for (int k = 0; k < N; k++) s.nzrows[k] = a.take<uint32_t>(s.dims[k]);
    s.nzcount = a.take<int64_t>(N);
    s.uni = a.take<double>((int64_t)N * 2 * J);
    s.samples = a.take<uint32_t>(J * N);
    s.weights = a.take<double>(J);
    s.d_owner = a.take<int32_t>(s.dtab);
    s.d_minj = a.take<int32_t>(s.dtab);
    s.d_count = a.take<int32_t>(s.dtab);
    s.slot_of = a.take<int32_t>(J);
    s.dkey = a.take<Key128>(J);
    s.flags = a.take<uint32_t>(J);
    s.sd = a.take<uint32_t>(J * N);
    s.wd = a.take<double>(J);
    s.counters = a.take<int64_t>(16);
    s.D = a.take<double>(J * R);
    s.part = a.take<double>(s.part_rows * P);
    s.dgram = a.take<double>(R2);
    s.dpinv = a.take<double>(R2);
    s.f_start = a.take<uint32_t>(J);
    s.f_len = a.take<uint32_t>(J);
    s.f_off = a.take<int64_t>(J);
    s.seg_start = a.take<int64_t>(I + 1);
    s.touched = a.take<uint32_t>(I);
    s.ugram = a.take<double>(R2);
    s.ngram = a.take<double>(R2);
    s.upinv = a.take<double>(R2);
    s.fitpart = a.take<double>(2 * 152 * 8);
    s.status = a.take<DeviceStatus>(1);
    s.scan_sc = a.take<char>((int64_t)scan_scratch_bytes(std::max(std::max(J, I), nnz)));
    s.dims_dev = a.take<int64_t>(kMaxModes);
    s.Mexact = a.take<double>(I * R);
    s.scal = a.take<double>(8);
    s.ex_j = a.take<uint32_t>(nnz);
    s.ex_val = a.take<double>(nnz);
    for (int b = 0; b < 2; b++) {
        s.hit_key[b] = a.take<uint32_t>(nnz);
        s.hit_pay[b] = a.take<uint32_t>(nnz);
        if (s.cfg.precision != EXAFAC_PREC_FP64) s.pay64[b] = a.take<uint64_t>(nnz);
    }
    s.os_status = a.take<uint64_t>(256 * (int64_t)hitsort_tile_stride(nnz));
    s.os_aux = a.take<uint32_t>(4 + 4 * 256 + 1);
    s.Mc = a.take<double>(I * std::max(R, 16));  // FP64 rows of R, or FP32 rows padded to a multiple of 4
    const int64_t chunks = ceil_div(nnz, kSegChunkF32) + 1;
    // carries (doubles): chunks of 64 hits x 32 columns (R <= 32), of 64 hits
    // x 32 ceil(R / 32) columns (R > 32, FP64 or FP32), or of 128 hits x
    // 32 ceil(R / 32) columns (the exact MTTKRP)
    const int64_t carry = std::max(chunks * (int64_t)(32 * ceil_div(R, 32)),
                                   (ceil_div(nnz, kSegChunkHits) + 1) * (int64_t)(32 * ceil_div(R, 32)));
    s.carry_first = a.take<double>(carry);
    s.carry_last = a.take<double>(carry);
    s.carry_row = a.take<uint32_t>(chunks);
    s.carry_seg = a.take<uint32_t>(chunks);
    s.chunk_seg = a.take<uint32_t>(chunks);
    s.expand_first = a.take<uint32_t>(ceil_div(nnz, kExpandChunk) + 1);
    const int64_t rs = std::max(32, f32_row_stride(R));  // FP32 rows padded to a multiple of 4 floats
    if (s.cfg.precision != EXAFAC_PREC_FP64) s.Uc = a.take<float>(I * rs);
    s.rowbits = a.take<uint32_t>(ceil_div(I, 32));
    s.Df = a.take<float>(J * rs);
}

static int plan(const exafac_als_config* cfg, Session& s) {
    EXAFAC_ARG(cfg != nullptr, "null config");
    EXAFAC_ARG(cfg->N >= 2 && cfg->N <= kMaxModes, "N must be in [2, 8]");
    EXAFAC_ARG(cfg->R >= 1 && cfg->R <= kMaxRank, "R must be in [1, 128]");
    EXAFAC_ARG(cfg->nnz >= 1 && cfg->nnz < (int64_t)0xffffffffll, "nnz must be in [1, 2^32 - 1)");
    EXAFAC_ARG(cfg->J_max >= 1 && cfg->J_max < ((int64_t)1 << 31), "J_max must be in [1, 2^31)");
    EXAFAC_ARG(cfg->sampler == EXAFAC_SAMPLER_CP_ARLS_LEV || cfg->sampler == EXAFAC_SAMPLER_STS_CP, "bad sampler");
    EXAFAC_ARG(cfg->precision == EXAFAC_PREC_FP64 || cfg->precision == EXAFAC_PREC_TF32 ||
                   cfg->precision == EXAFAC_PREC_BF16,
               "precision must be FP64, TF32 or BF16");
    EXAFAC_ARG(cfg->preprocessing >= 0 && cfg->preprocessing <= 2, "bad preprocessing");
    s.cfg = *cfg;
    s.N = cfg->N;
    s.R = cfg->R;
    s.P = packed_size(cfg->R);
    s.nnz = cfg->nnz;
    s.Jmax = cfg->J_max;
    s.Imax = 1;
    for (int k = 0; k < s.N; k++) {
        EXAFAC_ARG(cfg->dims[k] >= 1 && cfg->dims[k] <= (int64_t)0xffffffffll, "mode sizes must be in [1, 2^32)");
        s.dims[k] = cfg->dims[k];
        s.Imax = std::max(s.Imax, s.dims[k]);
    }
    for (int n = 0; n < s.N; n++) {
        Lookup& L = s.look[n];
        L.spec = make_keyspec(s.N, s.dims, n);
        EXAFAC_ARG(L.spec.bits <= 128, "packed coordinates exceed 128 bits");
        L.kw = L.spec.bits <= 64 ? 1 : 2;
        L.nslots = next_pow2(std::max<int64_t>(2 * s.nnz, 16));
    }
    for (int k = 0; k < s.N; k++) s.rtree[k] = make_tree_shape(s.dims[k], s.R);
    s.etree = make_tree_shape(s.R, 1);
    s.dtab = next_pow2(std::max<int64_t>(2 * s.Jmax, 16));
    // Gram partials: one per 32-row block of the row kernels, and one per CTA
    // of the tiled solve (152 * 2 CTAs).
    s.part_rows = std::max<int64_t>(ceil_div(std::max(s.Jmax, s.Imax), 32), 1024);
    return EXAFAC_OK;
}

static int check_status(Session& s, cudaStream_t st) {
    DeviceStatus h;
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(&h, s.status, sizeof(h), cudaMemcpyDeviceToHost, st));
    EXAFAC_CUDA_TRY(cudaStreamSynchronize(st));
    if (h.code != EXAFAC_OK) {
        char buf[160];
        snprintf(buf, sizeof(buf), "device check failed at site %d: value %lld, bound %lld", h.where, h.a, h.b);
        set_error(buf);
        return h.code;
    }
    return EXAFAC_OK;
}

// Sampler update for mode k (CP_ARLS_LEV::update_sampler cp_arls_lev.hpp:25-34,
// STS_CP::update_sampler sts_cp.hpp:63-65).  ngram holds the normalised Gram.
static int refresh_sampler(Session& s, int k, bool all_rows, cudaStream_t st) {
    const int R = s.R;
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.gram + (int64_t)k * R * R, s.ngram, sizeof(double) * R * R,
                                    cudaMemcpyDeviceToDevice, st));
    if (s.cfg.sampler == EXAFAC_SAMPLER_CP_ARLS_LEV) {
        EXAFAC_TRY(launch_pinv(R, s.ngram, s.upinv, 1e-11, s.vt, st));
        if (all_rows) EXAFAC_CUDA_TRY(cudaMemsetAsync(s.scores[k], 0, sizeof(double) * s.dims[k], st));
        EXAFAC_TRY(arls_leverage(s, k, all_rows, s.upinv, st));
        EXAFAC_TRY(arls_build_cdf(s, k, nullptr, nullptr, st));
    } else {
        EXAFAC_TRY(launch_tree_build(s.rtree[k], R, s.F.U[k], s.treeG[k], st));
        EXAFAC_TRY(sts_refresh_f32(s, k, st));
    }
    return EXAFAC_OK;
}

// Gram of every factor over all rows into s.gram (fit, exact ALS).
static int all_grams(Session& s, cudaStream_t st) {
    for (int k = 0; k < s.N; k++)
        EXAFAC_TRY(gram_rows(s, s.F.U[k], s.dims[k], nullptr, nullptr, s.gram + (int64_t)k * s.R * s.R, st));
    return EXAFAC_OK;
}

static int draw_into_session(Session& s, int n, int64_t J, const double* uni, const uint32_t* perms, cudaStream_t st) {
    const bool sts = s.cfg.sampler == EXAFAC_SAMPLER_STS_CP;
    if (uni == nullptr) {
        EXAFAC_TRY(gen_uniforms(s, s.uni, (int64_t)s.N * (sts ? 2 : 1) * J, st));
        uni = s.uni;
    }
    if (sts) {
        EXAFAC_TRY(sts_compute_M(s, n, st));
        EXAFAC_TRY(sts_draw(s, n, J, uni, st));
    } else {
        EXAFAC_TRY(arls_draw(s, n, J, uni, perms, st));
    }
    return EXAFAC_OK;
}

}  // namespace exafac

using namespace exafac;

struct exafac_als_s {
    Session s;
    // Region timing (als_optimizer.hpp:19-27): events at the region borders
    // of each step, read back at the end of the step when enabled.
    // Each timed step takes a set of six events from a pool and records its
    // region borders into it; nothing waits for them until the times are read
    // (exafac_als_region_times), or until more than kMaxPendingSteps steps are
    // pending, when the oldest are drained.
    static constexpr size_t kMaxPendingSteps = 512;
    struct EventSet {
        cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    };
    bool timing = false;
    std::vector<EventSet> free_sets;
    std::deque<EventSet> pending;
    EventSet* cur = nullptr;
    double region[7] = {0, 0, 0, 0, 0, 0, 0};
    // Side stream for the design rows, their Gram and its pseudo-inverse,
    // which run beside the fiber lookup and the hit sort (fork / join events
    // on the caller's stream).
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // recorded on the side stream once the design rows are written (before
    // their Gram's pseudo-inverse): the wide MTTKRP needs the rows only, the
    // solve after it the pseudo-inverse (join)
    cudaEvent_t rows_ready = nullptr;
    // and, queued after it, the clearing of the factor rows the previous
    // update of the mode wrote and this one does not (disjoint from the rows
    // the update writes), beside the MTTKRP and solve; joined before the
    // renormalisation
    cudaEvent_t fork2 = nullptr, join2 = nullptr;
    // One captured sweep (exafac_als_sweeps), keyed by J and the uniforms
    // pointer it was captured with, and the kernels it launches.
    cudaStream_t cap = nullptr;
    cudaEvent_t cap_ev = nullptr;
    cudaGraphExec_t sweep_exec = nullptr;
    int64_t sweep_J = -1;
    const double* sweep_uni = nullptr;
    long long sweep_launches = 0;
    ~exafac_als_s() {
        for (auto* list : {&free_sets})
            for (auto& set : *list)
                for (auto& e : set.ev)
                    if (e) cudaEventDestroy(e);
        for (auto& set : pending)
            for (auto& e : set.ev)
                if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (rows_ready) cudaEventDestroy(rows_ready);
        if (fork2) cudaEventDestroy(fork2);
        if (join2) cudaEventDestroy(join2);
        if (side) cudaStreamDestroy(side);
        if (sweep_exec) cudaGraphExecDestroy(sweep_exec);
        if (cap_ev) cudaEventDestroy(cap_ev);
        if (cap) cudaStreamDestroy(cap);
    }
};

// Launches the design rows, their Gram and its pseudo-inverse on the side
// stream after the work already queued on st (the deduplicated samples):
// they need nothing of the fibre lookup and hit grouping that st runs next,
// and those write nothing they read.  st must wait on h->rows_ready before
// reading the design rows and on h->join before reading the pseudo-inverse.
static int fork_design(exafac_als_s* h, int n, int64_t J, cudaStream_t st) {
    if (!h->side) {
        EXAFAC_CUDA_TRY(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        EXAFAC_CUDA_TRY(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
        EXAFAC_CUDA_TRY(cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming));
        EXAFAC_CUDA_TRY(cudaEventCreateWithFlags(&h->rows_ready, cudaEventDisableTiming));
        EXAFAC_CUDA_TRY(cudaEventCreateWithFlags(&h->fork2, cudaEventDisableTiming));
        EXAFAC_CUDA_TRY(cudaEventCreateWithFlags(&h->join2, cudaEventDisableTiming));
    }
    EXAFAC_CUDA_TRY(cudaEventRecord(h->fork, st));
    EXAFAC_CUDA_TRY(cudaStreamWaitEvent(h->side, h->fork, 0));
    EXAFAC_TRY(design_gram(h->s, n, J, h->side));
    EXAFAC_CUDA_TRY(cudaEventRecord(h->rows_ready, h->side));
    EXAFAC_TRY(design_pinv(h->s, h->side));
    EXAFAC_CUDA_TRY(cudaEventRecord(h->join, h->side));
    return EXAFAC_OK;
}

// Adds the region times of the oldest pending step (waits for its last event).
static int drain_one(exafac_als_s* h) {
    exafac_als_s::EventSet set = h->pending.front();
    h->pending.pop_front();
    h->free_sets.push_back(set);
    EXAFAC_CUDA_TRY(cudaEventSynchronize(set.ev[5]));
    const int map[5] = {0, 2, 3, 5, 6};  // R1, R3, R4, R6, R7
    float ms[5];
    for (int i = 0; i < 5; i++) {
        // A step that returned an error part way left later borders
        // unrecorded: it adds nothing.
        if (cudaEventElapsedTime(&ms[i], set.ev[i], set.ev[i + 1]) != cudaSuccess) {
            (void)cudaGetLastError();
            return EXAFAC_OK;
        }
    }
    for (int i = 0; i < 5; i++) h->region[map[i]] += ms[i] * 1e-3;
    return EXAFAC_OK;
}

static int drain_all(exafac_als_s* h) {
    while (!h->pending.empty()) EXAFAC_TRY(drain_one(h));
    return EXAFAC_OK;
}

// Region border i of the current step (0 opens the step, 5 closes it).
static int mark(exafac_als_s* h, int i, cudaStream_t st) {
    if (!h->timing) return EXAFAC_OK;
    if (i == 0) {
        if (h->pending.size() >= exafac_als_s::kMaxPendingSteps) EXAFAC_TRY(drain_one(h));
        exafac_als_s::EventSet set;
        if (!h->free_sets.empty()) {
            set = h->free_sets.back();
            h->free_sets.pop_back();
        } else {
            for (auto& e : set.ev) EXAFAC_CUDA_TRY(cudaEventCreate(&e));
        }
        h->pending.push_back(set);
        h->cur = &h->pending.back();
    }
    EXAFAC_CUDA_TRY(cudaEventRecord(h->cur->ev[i], st));
    return EXAFAC_OK;
}

extern "C" int exafac_als_enable_timing(exafac_als_t h, int32_t enable) {
    EXAFAC_ARG(h != nullptr, "null session");
    // steps timed before this call no longer count
    while (!h->pending.empty()) {
        h->free_sets.push_back(h->pending.front());
        h->pending.pop_front();
    }
    h->cur = nullptr;
    h->timing = enable != 0;
    for (double& r : h->region) r = 0.0;
    return EXAFAC_OK;
}

extern "C" int exafac_als_region_times(exafac_als_t h, double* out7) {
    EXAFAC_ARG(h != nullptr && out7 != nullptr, "null argument");
    EXAFAC_TRY(drain_all(h));
    for (int i = 0; i < 7; i++) out7[i] = h->region[i];
    return EXAFAC_OK;
}

extern "C" const char* exafac_last_error(void) { return g_last_error.c_str(); }
extern "C" int exafac_abi_version(void) { return EXAFAC_ABI_VERSION; }
extern "C" long long exafac_kernel_launches(void) { return g_launches.load(); }

extern "C" int exafac_als_workspace_size(const exafac_als_config* cfg, size_t* persistent_bytes, size_t* setup_b) {
    Session s;
    EXAFAC_TRY(plan(cfg, s));
    s.arena = Arena();
    carve(s);
    if (persistent_bytes) *persistent_bytes = s.arena.used + 256;
    if (setup_b) *setup_b = setup_bytes(s) + 256;
    return EXAFAC_OK;
}

extern "C" int exafac_als_create(const exafac_als_config* cfg, void* persistent, size_t bytes, exafac_als_t* out) {
    EXAFAC_ARG(out != nullptr && persistent != nullptr, "null argument");
    EXAFAC_ARG(((uintptr_t)persistent & 255) == 0, "workspace must be 256-byte aligned");
    exafac_als_s* h = new (std::nothrow) exafac_als_s();
    if (!h) {
        set_error("out of host memory");
        return EXAFAC_ERR_ARG;
    }
    int rc = plan(cfg, h->s);
    if (rc != EXAFAC_OK) {
        delete h;
        return rc;
    }
    h->s.arena.base = reinterpret_cast<char*>(persistent);
    h->s.arena.cap = bytes;
    carve(h->s);
    if (h->s.arena.overflow) {
        delete h;
        set_error("exafac_als_create: workspace smaller than exafac_als_workspace_size");
        return EXAFAC_ERR_WORKSPACE;
    }
    *out = h;
    return EXAFAC_OK;
}

extern "C" int exafac_als_destroy(exafac_als_t h) {
    delete h;
    return EXAFAC_OK;
}

extern "C" int exafac_als_set_seed(exafac_als_t h, uint64_t seed) {
    EXAFAC_ARG(h != nullptr, "null session");
    h->s.seed = seed;
    if (h->sweep_exec) {  // the captured sweep holds the old key
        cudaGraphExecDestroy(h->sweep_exec);
        h->sweep_exec = nullptr;
    }
    if (h->s.counters)  // restart the stream (synchronous; a set-up call)
        EXAFAC_CUDA_TRY(cudaMemset(h->s.counters + kRngSlot, 0, sizeof(int64_t)));
    return EXAFAC_OK;
}

extern "C" int exafac_als_init(exafac_als_t h, const uint32_t* idx, const double* vals, const exafac_factors* F,
                               void* setup, size_t setup_sz, double* tensor_norm, void* stream) {
    EXAFAC_ARG(h && idx && vals && F && setup, "null argument");
    Session& s = h->s;
    if (h->sweep_exec) {  // the captured sweep holds the previous factor pointers
        cudaGraphExecDestroy(h->sweep_exec);
        h->sweep_exec = nullptr;
    }
    cudaStream_t st = (cudaStream_t)stream;
    for (int k = 0; k < s.N; k++) EXAFAC_ARG(F->U[k] != nullptr, "null factor matrix");
    EXAFAC_ARG(F->sigma != nullptr, "null sigma");
    s.F = *F;
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.status, 0, sizeof(DeviceStatus), st));
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.counters, 0, sizeof(int64_t) * 16, st));
    // look-back status words carry an epoch (counters[kSortEpochSlot]); both start at zero
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.os_status, 0, sizeof(uint64_t) * 256 * hitsort_tile_stride(s.nnz), st));
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.dims_dev, s.dims, sizeof(int64_t) * kMaxModes, cudaMemcpyHostToDevice, st));
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.idx, idx, sizeof(uint32_t) * s.nnz * s.N, cudaMemcpyDeviceToDevice, st));
    EXAFAC_TRY(preprocess_values(s, vals, st));
    for (int n = 0; n < s.N; n++) EXAFAC_TRY(build_lookup(s, n, setup, setup_sz, st));
    // Sampler construction over the initial (dense) factors.
    for (int k = 0; k < s.N; k++) {
        EXAFAC_TRY(gram_rows(s, s.F.U[k], s.dims[k], nullptr, nullptr, s.ugram, st));
        // The factors are used as given: their Gram is the sampler's Gram.
        EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.ngram, s.ugram, sizeof(double) * s.R * s.R, cudaMemcpyDeviceToDevice, st));
        EXAFAC_TRY(refresh_sampler(s, k, true, st));
        s.dense[k] = true;
    }
    double normsq = 0.0;
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(&normsq, s.scal + 0, sizeof(double), cudaMemcpyDeviceToHost, st));
    EXAFAC_TRY(check_status(s, st));
    s.tensor_norm = std::sqrt(normsq);
    if (tensor_norm) *tensor_norm = s.tensor_norm;
    s.initialized = true;
    return EXAFAC_OK;
}

extern "C" int exafac_als_draw(exafac_als_t h, int32_t mode, int64_t J, const double* uni, const uint32_t* perms,
                               uint32_t* samples_out, double* weights_out, void* stream) {
    EXAFAC_ARG(h && h->s.initialized, "session not initialised");
    Session& s = h->s;
    EXAFAC_ARG(mode >= 0 && mode < s.N, "mode out of range");
    EXAFAC_ARG(J >= 1 && J <= s.Jmax, "J out of range");
    cudaStream_t st = (cudaStream_t)stream;
    EXAFAC_TRY(draw_into_session(s, mode, J, uni, perms, st));
    if (samples_out)
        EXAFAC_CUDA_TRY(
            cudaMemcpyAsync(samples_out, s.samples, sizeof(uint32_t) * J * s.N, cudaMemcpyDeviceToDevice, st));
    if (weights_out)
        EXAFAC_CUDA_TRY(cudaMemcpyAsync(weights_out, s.weights, sizeof(double) * J, cudaMemcpyDeviceToDevice, st));
    return EXAFAC_OK;
}

extern "C" int exafac_als_step(exafac_als_t h, int32_t n, int64_t J, const double* uni, const uint32_t* perms,
                               void* stream) {
    EXAFAC_ARG(h && h->s.initialized, "session not initialised");
    Session& s = h->s;
    EXAFAC_ARG(n >= 0 && n < s.N, "mode out of range");
    EXAFAC_ARG(J >= 1 && J <= s.Jmax, "J out of range");
    cudaStream_t st = (cudaStream_t)stream;
    EXAFAC_TRY(mark(h, 0, st));
    // R1: samples and weights.
    EXAFAC_TRY(draw_into_session(s, n, J, uni, perms, st));
    EXAFAC_TRY(mark(h, 1, st));
    // R2 (row gather) is a no-op on one GPU: factors are read in place.
    // R3: deduplicate; the design rows, Gram and pseudo-inverse go to the
    // side stream.
    EXAFAC_TRY(dedup(s, n, J, st));
    EXAFAC_TRY(fork_design(h, n, J, st));
    EXAFAC_TRY(mark(h, 2, st));
    // R4: fiber lookup, hits grouped by output row, MTTKRP rows, then
    // U = MTTKRP * Phi on the touched rows (the other rows are zero).
    const bool arls = s.cfg.sampler == EXAFAC_SAMPLER_CP_ARLS_LEV;
    const bool tiled = s.R <= 32;
    EXAFAC_TRY(lookup_hits(s, n, J, s.cfg.precision != EXAFAC_PREC_FP64, st));
    // rowbits is set: the old rows are cleared on the side stream
    EXAFAC_CUDA_TRY(cudaEventRecord(h->fork2, st));
    EXAFAC_CUDA_TRY(cudaStreamWaitEvent(h->side, h->fork2, 0));
    EXAFAC_TRY(zero_old_rows(s, n, h->side));
    EXAFAC_CUDA_TRY(cudaEventRecord(h->join2, h->side));
    if (tiled) {
        EXAFAC_CUDA_TRY(cudaStreamWaitEvent(st, h->join, 0));
        EXAFAC_TRY(mttkrp_solve_balanced(s, n, st));
    } else {
        // the MTTKRP rows beside the pseudo-inverse, which only the solve reads
        EXAFAC_CUDA_TRY(cudaStreamWaitEvent(st, h->rows_ready, 0));
        EXAFAC_TRY(mttkrp_solve_wide(s, n, st, h->join));
    }
    // the old rows are cleared (the renormalisation may rescale every row)
    EXAFAC_CUDA_TRY(cudaStreamWaitEvent(st, h->join2, 0));
    EXAFAC_TRY(mark(h, 3, st));
    // R5 (dense reduce) is empty at one rank.  R6: renormalise (and, for
    // CP-ARLS-LEV, the new leverage scores of the touched rows).
    if (tiled) EXAFAC_TRY(normalize_balanced(s, n, arls, st));
    else EXAFAC_TRY(normalize_wide(s, n, arls, st));
    EXAFAC_TRY(mark(h, 4, st));
    // R7: sampler update (CDF of the new scores, or the row tree).
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.gram + (int64_t)n * s.R * s.R, s.ngram, sizeof(double) * s.R * s.R,
                                    cudaMemcpyDeviceToDevice, st));
    if (arls) EXAFAC_TRY(arls_build_cdf(s, n, s.touched, s.counters + 2, st));
    else EXAFAC_TRY(sts_rebuild_tree(s, n, st));
    EXAFAC_TRY(keep_touched(s, n, st));
    s.dense[n] = false;
    EXAFAC_TRY(mark(h, 5, st));
    return EXAFAC_OK;
}

// One sweep: steps 0..N-1; explicit uniforms are N per-step blocks.
static int run_sweep(exafac_als_s* h, int64_t J, const double* uni, cudaStream_t st) {
    const Session& s = h->s;
    const int64_t per_step = (int64_t)s.N * (s.cfg.sampler == EXAFAC_SAMPLER_STS_CP ? 2 : 1) * J;
    for (int n = 0; n < s.N; n++) EXAFAC_TRY(exafac_als_step(h, n, J, uni ? uni + n * per_step : nullptr, nullptr, st));
    return EXAFAC_OK;
}

static bool any_dense(const Session& s) {
    for (int k = 0; k < s.N; k++)
        if (s.dense[k]) return true;
    return false;
}

// Captures one steady-state sweep into s->sweep_exec on the internal stream
// (ordered after the work already queued on st).
static int capture_sweep(exafac_als_s* h, int64_t J, const double* uni, cudaStream_t st) {
    if (h->sweep_exec) {
        cudaGraphExecDestroy(h->sweep_exec);
        h->sweep_exec = nullptr;
    }
    if (!h->cap) {
        EXAFAC_CUDA_TRY(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
        EXAFAC_CUDA_TRY(cudaEventCreateWithFlags(&h->cap_ev, cudaEventDisableTiming));
    }
    EXAFAC_CUDA_TRY(cudaEventRecord(h->cap_ev, st));
    EXAFAC_CUDA_TRY(cudaStreamWaitEvent(h->cap, h->cap_ev, 0));
    const long long l0 = exafac_kernel_launches();
    EXAFAC_CUDA_TRY(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeRelaxed));
    const int rc = run_sweep(h, J, uni, h->cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->cap, &graph);
    h->sweep_launches = exafac_kernel_launches() - l0;
    add_launches(-h->sweep_launches);  // recorded, not launched
    if (rc != EXAFAC_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    EXAFAC_CUDA_TRY(e);
    const cudaError_t ei = cudaGraphInstantiate(&h->sweep_exec, graph, 0);
    cudaGraphDestroy(graph);
    EXAFAC_CUDA_TRY(ei);
    h->sweep_J = J;
    h->sweep_uni = uni;
    return EXAFAC_OK;
}

extern "C" int exafac_als_sweeps(exafac_als_t h, int64_t J, int32_t count, const double* uni, void* stream) {
    EXAFAC_ARG(h && h->s.initialized, "session not initialised");
    Session& s = h->s;
    EXAFAC_ARG(J >= 1 && J <= s.Jmax, "J out of range");
    EXAFAC_ARG(count >= 0, "count must be >= 0");
    EXAFAC_ARG(!h->timing, "exafac_als_sweeps: region timing is on (region borders are recorded by exafac_als_step)");
    cudaStream_t st = (cudaStream_t)stream;
    int done = 0;
    // A factor that no sampled step has updated yet is cleared whole by its
    // next update, a different launch sequence: run plain sweeps until none is.
    while (done < count && any_dense(s)) {
        EXAFAC_TRY(run_sweep(h, J, uni, st));
        done++;
    }
    if (done == count) return EXAFAC_OK;
    if (!h->sweep_exec || h->sweep_J != J || h->sweep_uni != uni) EXAFAC_TRY(capture_sweep(h, J, uni, st));
    for (; done < count; done++) {
        EXAFAC_CUDA_TRY(cudaGraphLaunch(h->sweep_exec, st));
        add_launches(h->sweep_launches);
    }
    return EXAFAC_OK;
}

extern "C" int exafac_als_sampled_mttkrp(exafac_als_t h, int32_t n, int64_t Ju, const uint32_t* samples,
                                         const double* design, double* out, void* stream) {
    EXAFAC_ARG(h && h->s.initialized, "session not initialised");
    Session& s = h->s;
    EXAFAC_ARG(n >= 0 && n < s.N, "mode out of range");
    EXAFAC_ARG(Ju >= 0 && Ju <= s.Jmax, "sample count out of range");
    EXAFAC_ARG(out && (Ju == 0 || (samples && design)), "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.counters + 0, &Ju, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    if (Ju > 0) {
        EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.sd, samples, sizeof(uint32_t) * Ju * s.N, cudaMemcpyDeviceToDevice, st));
        EXAFAC_CUDA_TRY(cudaMemcpyAsync(s.D, design, sizeof(double) * Ju * s.R, cudaMemcpyDeviceToDevice, st));
    }
    EXAFAC_TRY(lookup_hits(s, n, std::max<int64_t>(Ju, 1), false, st));
    EXAFAC_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * s.dims[n] * s.R, st));
    if (s.R <= 32) EXAFAC_TRY(mttkrp_scatter_out(s, out, st));
    else EXAFAC_TRY(spmm_solve_into(s, n, nullptr, out, st));
    // The host value of Ju above must outlive the async copy.
    EXAFAC_CUDA_TRY(cudaStreamSynchronize(st));
    return EXAFAC_OK;
}

extern "C" int exafac_als_exact_step(exafac_als_t h, int32_t n, void* stream) {
    EXAFAC_ARG(h && h->s.initialized, "session not initialised");
    Session& s = h->s;
    EXAFAC_ARG(n >= 0 && n < s.N, "mode out of range");
    cudaStream_t st = (cudaStream_t)stream;
    const int R = s.R;
    EXAFAC_TRY(all_grams(s, st));
    EXAFAC_TRY(chain_gram(s, n, s.dgram, st));
    EXAFAC_TRY(launch_pinv(R, s.dgram, s.dpinv, 1e-11, s.vt, st));
    EXAFAC_TRY(exact_mttkrp(s, n, s.Mexact, st));
    EXAFAC_TRY(matmul_rows_sym(s, s.Mexact, s.dpinv, s.F.U[n], s.dims[n], st));
    EXAFAC_TRY(normalize_factor(s, n, true, st));
    s.dense[n] = true;
    EXAFAC_TRY(refresh_sampler(s, n, true, st));
    return EXAFAC_OK;
}

__global__ void fit_finish_kernel(int R, const double* __restrict__ chain, const double* __restrict__ sigma,
                                  double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double acc = 0.0;
    for (int i = 0; i < R; i++)
        for (int j = 0; j < R; j++) acc += chain[i * R + j] * sigma[i] * sigma[j];
    *out = acc;
}

extern "C" int exafac_als_fit(exafac_als_t h, double* fit, void* stream) {
    EXAFAC_ARG(h && h->s.initialized && fit, "session not initialised");
    Session& s = h->s;
    cudaStream_t st = (cudaStream_t)stream;
    EXAFAC_TRY(all_grams(s, st));
    EXAFAC_TRY(chain_gram(s, -1, s.dgram, st));
    fit_finish_kernel<<<1, 32, 0, st>>>(s.R, s.dgram, s.F.sigma, s.scal + 1); count_launch();
    EXAFAC_CHECK_LAUNCH();
    EXAFAC_TRY(fit_residual(s, s.scal + 2, st));
    double v[2];
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(v, s.scal + 1, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
    EXAFAC_TRY(check_status(s, st));
    *fit = 1.0 - std::sqrt(v[0] + v[1]) / s.tensor_norm;
    return EXAFAC_OK;
}

extern "C" int exafac_als_set_wait_limit(exafac_als_t h, uint32_t polls, int64_t withhold_tile) {
    EXAFAC_ARG(h != nullptr, "null session");
    EXAFAC_ARG(withhold_tile >= -1, "withhold_tile must be -1 (off) or a tile index");
    h->s.wait_polls = polls == 0 ? kSpinLimit : polls;
    h->s.withhold_tile = withhold_tile;
    if (h->sweep_exec) {  // the captured sweep holds the old limits
        cudaGraphExecDestroy(h->sweep_exec);
        h->sweep_exec = nullptr;
    }
    return EXAFAC_OK;
}

extern "C" int exafac_als_estimated_fit(exafac_als_t h, int64_t Z, const uint32_t* zero_idx, uint64_t seed,
                                        double* fit, int64_t* kept, void* stream) {
    EXAFAC_ARG(h && h->s.initialized, "session not initialised");
    Session& s = h->s;
    cudaStream_t st = (cudaStream_t)stream;
    EXAFAC_TRY(estimated_fit(s, Z, zero_idx, seed, fit, kept, st));
    return check_status(s, st);
}

extern "C" int exafac_als_step_info(exafac_als_t h, exafac_step_info* out, void* stream) {
    EXAFAC_ARG(h && out, "null argument");
    Session& s = h->s;
    cudaStream_t st = (cudaStream_t)stream;
    int64_t c[16];
    DeviceStatus ds;
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(c, s.counters, sizeof(c), cudaMemcpyDeviceToHost, st));
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(&ds, s.status, sizeof(ds), cudaMemcpyDeviceToHost, st));
    EXAFAC_CUDA_TRY(cudaStreamSynchronize(st));
    out->unique_samples = c[0];
    out->hits = c[1];
    out->touched_rows = c[2];
    out->hits_total = c[5];
    out->device_status = ds.code;
    out->pad = 0;
    return EXAFAC_OK;
}

extern "C" int exafac_als_last_dedup(exafac_als_t h, const uint32_t** samples, const double** weights,
                                     const double** gram, const double** pinv) {
    EXAFAC_ARG(h != nullptr, "null session");
    Session& s = h->s;
    if (samples) *samples = s.sd;
    if (weights) *weights = s.wd;
    if (gram) *gram = s.dgram;
    if (pinv) *pinv = s.dpinv;
    return EXAFAC_OK;
}
