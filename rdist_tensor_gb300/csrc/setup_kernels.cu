// Set-up: value preprocessing (SparseTensor ctor, sparse_tensor.hpp:36-75) and
// the per-mode sorted copies with their fiber hash tables
// (AccumulatorStationary::initialize_ground_truth_for_als + SortIdxLookup ctor,
// accumulator_stationary.hpp:38-137, sort_lookup.hpp:37-102).
#include "engine.cuh"
#include "prims.cuh"

namespace exafac {

__global__ void preprocess_kernel(int64_t nnz, int mode, const double* __restrict__ in, double* __restrict__ out,
                                  double* __restrict__ part) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        double v = in[i];
        if (mode == EXAFAC_PRE_LOG_COUNT) v = log(v + 1);
        else if (mode == EXAFAC_PRE_ONES) v = 1.0;
        out[i] = v;
        acc += v * v;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_parts_kernel(const double* __restrict__ part, int n, double* __restrict__ out) {
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

int preprocess_values(Session& s, const double* vals_in, cudaStream_t st) {
    const int blocks = 152 * 8;
    preprocess_kernel<<<blocks, 256, 0, st>>>(s.nnz, s.cfg.preprocessing, vals_in, s.vals, s.fitpart); count_launch();
    sum_parts_kernel<<<1, 256, 0, st>>>(s.fitpart, blocks, s.scal + 0); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

__global__ void pack_keys_kernel(KeySpec spec, int64_t nnz, const uint32_t* __restrict__ idx, uint64_t* __restrict__ lo,
                                 uint64_t* __restrict__ hi, uint32_t* __restrict__ pay, DeviceStatus* status,
                                 const int64_t* __restrict__ dims) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t* c = idx + i * spec.N;
        for (int k = 0; k < spec.N; k++)
            if ((int64_t)c[k] >= dims[k]) report(status, EXAFAC_ERR_DEVICE, 10, c[k], dims[k]);
        Key128 key = pack_key(spec, c);
        lo[i] = key.lo;
        if (hi) hi[i] = key.hi;
        pay[i] = (uint32_t)i;
    }
}

__global__ void gather_sorted_kernel(int N, int n, int64_t nnz, const uint32_t* __restrict__ pay,
                                     const uint32_t* __restrict__ idx, const double* __restrict__ vals,
                                     uint32_t* __restrict__ rows_n, double* __restrict__ vals_n) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = pay[p];
        rows_n[p] = idx[i * N + n];
        vals_n[p] = vals[i];
    }
}

__global__ void fiber_flag_kernel(int64_t nnz, const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi,
                                  uint32_t* __restrict__ flag) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
        bool b = p == 0 || lo[p] != lo[p - 1] || (hi && hi[p] != hi[p - 1]);
        flag[p] = b ? 1u : 0u;
    }
}

__global__ void fiber_compact_kernel(int64_t nnz, const uint32_t* __restrict__ flag, const int64_t* __restrict__ fid,
                                     uint32_t* __restrict__ fstart, const int64_t* __restrict__ nf) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
        if (flag[p]) fstart[fid[p]] = (uint32_t)p;
    if (blockIdx.x == 0 && threadIdx.x == 0) fstart[*nf] = (uint32_t)nnz;
}

template <typename Slot>
__device__ __forceinline__ void slot_fill(Slot& sl, uint64_t lo, uint64_t hi, uint32_t len);
template <>
__device__ __forceinline__ void slot_fill<Slot1>(Slot1& sl, uint64_t lo, uint64_t, uint32_t len) {
    sl.key = lo;
    sl.len = len;
}
template <>
__device__ __forceinline__ void slot_fill<Slot2>(Slot2& sl, uint64_t lo, uint64_t hi, uint32_t len) {
    sl.lo = lo;
    sl.hi = hi;
    sl.len = len;
}

template <typename Slot>
__global__ void fiber_insert_kernel(const int64_t* __restrict__ nf_dev, const uint32_t* __restrict__ fstart,
                                    const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi, Slot* slots,
                                    int64_t mask, DeviceStatus* status) {
    const int64_t nf = *nf_dev;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t start = fstart[f];
        const uint32_t len = fstart[f + 1] - start;
        Key128 key{lo[start], hi ? hi[start] : 0ull};
        int64_t h = (int64_t)(hash_key(key) & (uint64_t)mask);
        bool placed = false;
        for (int64_t probe = 0; probe <= mask; probe++) {
            if (atomicCAS(&slots[h].start, kEmpty, start) == kEmpty) {
                slot_fill(slots[h], key.lo, key.hi, len);
                placed = true;
                break;
            }
            h = (h + 1) & mask;
        }
        if (!placed) report(status, EXAFAC_ERR_DEVICE, 11, f, mask + 1);
    }
}

struct SetupBufs {
    uint64_t *lo, *hi, *lo_s, *hi_s, *lo_t, *hi_t;
    uint32_t *pay, *pay_s, *pay_t, *flag, *fstart;
    int64_t *fid, *nf;
    void* scan_sc;
    void* radix_sc;
};

static size_t carve_setup(const Session& s, char* base, SetupBufs* b) {
    Arena a;
    a.base = base;
    a.cap = base ? (size_t)-1 : 0;
    const int64_t n = s.nnz;
    SetupBufs t;
    t.lo = a.take<uint64_t>(n);
    t.hi = a.take<uint64_t>(n);
    t.lo_s = a.take<uint64_t>(n);
    t.hi_s = a.take<uint64_t>(n);
    t.lo_t = a.take<uint64_t>(n);
    t.hi_t = a.take<uint64_t>(n);
    t.pay = a.take<uint32_t>(n);
    t.pay_s = a.take<uint32_t>(n);
    t.pay_t = a.take<uint32_t>(n);
    t.flag = a.take<uint32_t>(n);
    t.fstart = a.take<uint32_t>(n + 1);
    t.fid = a.take<int64_t>(n);
    t.nf = a.take<int64_t>(4);
    t.scan_sc = a.take<char>((int64_t)scan_scratch_bytes(n));
    t.radix_sc = a.take<char>((int64_t)radix_scratch_bytes(n));
    if (b) *b = t;
    return a.used;
}

size_t setup_bytes(const Session& s) { return carve_setup(s, nullptr, nullptr); }

int build_lookup(Session& s, int n, void* setup, size_t setup_sz, cudaStream_t st) {
    if (setup_sz < setup_bytes(s)) {
        set_error("exafac_als_init: setup workspace too small");
        return EXAFAC_ERR_WORKSPACE;
    }
    SetupBufs b;
    carve_setup(s, reinterpret_cast<char*>(setup), &b);
    Lookup& L = s.look[n];
    const int64_t nnz = s.nnz;
    const int kw = L.kw;
    const int blocks = 152 * 8;
    pack_keys_kernel<<<blocks, 256, 0, st>>>(L.spec, nnz, s.idx, b.lo, kw == 2 ? b.hi : nullptr, b.pay, s.status,
                                             s.dims_dev); count_launch();
    EXAFAC_CHECK_LAUNCH();
    EXAFAC_TRY(radix_sort_pairs(nnz, L.spec.bits, kw, b.lo, b.hi, b.pay, b.lo_s, b.hi_s, b.pay_s, b.lo_t, b.hi_t,
                                b.pay_t, b.radix_sc, st));
    gather_sorted_kernel<<<blocks, 256, 0, st>>>(s.N, n, nnz, b.pay_s, s.idx, s.vals, L.rows, L.vals); count_launch();
    fiber_flag_kernel<<<blocks, 256, 0, st>>>(nnz, b.lo_s, kw == 2 ? b.hi_s : nullptr, b.flag); count_launch();
    EXAFAC_CHECK_LAUNCH();
    EXAFAC_TRY(scan_exclusive_u32_to_i64(b.flag, b.fid, nnz, b.nf, b.scan_sc, st));
    fiber_compact_kernel<<<blocks, 256, 0, st>>>(nnz, b.flag, b.fid, b.fstart, b.nf); count_launch();
    EXAFAC_CHECK_LAUNCH();
    const size_t slot_bytes = kw == 1 ? sizeof(Slot1) : sizeof(Slot2);
    EXAFAC_CUDA_TRY(cudaMemsetAsync(L.slots, 0xff, slot_bytes * (size_t)L.nslots, st));
    count_launch();
    if (kw == 1)
        fiber_insert_kernel<Slot1><<<blocks, 256, 0, st>>>(b.nf, b.fstart, b.lo_s, nullptr, (Slot1*)L.slots,
                                                           L.nslots - 1, s.status);
    else
        fiber_insert_kernel<Slot2><<<blocks, 256, 0, st>>>(b.nf, b.fstart, b.lo_s, b.hi_s, (Slot2*)L.slots,
                                                           L.nslots - 1, s.status);
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

}  // namespace exafac
