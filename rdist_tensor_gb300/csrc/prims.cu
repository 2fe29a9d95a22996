// Device-wide scans (three-phase: block sums, scan of block sums, block-local
// scan plus carry) and a stable LSD radix sort used to build the per-mode
// sorted copies at set-up.
#include "prims.cuh"

namespace exafac {

constexpr int kScanThreads = 256;
constexpr int kScanItems = kScanTile / kScanThreads;  // 16

template <typename T>
__device__ T block_reduce_sum(T v, T* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w] = v;
    __syncthreads();
    T r = 0;
    if (threadIdx.x < 32) {
        r = (lane < (int)(blockDim.x >> 5)) ? red[lane] : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// Exclusive block scan of one value per thread; returns the prefix, *total = block sum.
template <typename T>
__device__ T block_exclusive_scan(T v, T* red, T* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) red[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        T x = lane < nw ? red[lane] : T(0);
        T xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += y;
        }
        if (lane < nw) red[lane] = xi - x;
        if (lane == nw - 1) red[32] = xi;
    }
    __syncthreads();
    T out = red[w] + inc - v;
    *total = red[32];
    __syncthreads();
    return out;
}

// Optional forms: element g is in[gather[g]] when gather is given, and the
// length is min(n, *n_dev) when n_dev is given (n sizes the grid).
template <typename Tin, typename Tacc>
__global__ void scan_block_sums(const Tin* __restrict__ in, int64_t n, Tacc* __restrict__ partial,
                                const uint32_t* __restrict__ gather = nullptr, const int64_t* n_dev = nullptr) {
    __shared__ Tacc red[33];
    pdl_wait();
    pdl_trigger();
    if (n_dev) n = min(n, *n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    if (base >= n) {  // uniform per block
        if (threadIdx.x == 0) partial[blockIdx.x] = Tacc(0);
        return;
    }
    Tacc v[kScanItems];  // all of the thread's loads in flight before the first add
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int64_t g = base + threadIdx.x + k * kScanThreads;
        v[k] = g < n ? (Tacc)in[gather ? (int64_t)gather[g] : g] : Tacc(0);
    }
    Tacc acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) acc += v[k];
    Tacc s = block_reduce_sum(acc, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

template <typename Tacc>
__global__ void scan_partials_kernel(Tacc* partial, int64_t nb, Tacc* total) {
    __shared__ Tacc red[33];
    pdl_wait();
    pdl_trigger();
    Tacc carry = 0;
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        Tacc v = i < nb ? partial[i] : Tacc(0);
        Tacc tot;
        Tacc ex = block_exclusive_scan(v, red, &tot);
        if (i < nb) partial[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// kNormalize (inclusive double scans): out_i = S_i / S_{n-1}, out_{n-1} = 1.
// The tile is held in shared memory with one pad word after every 16
// elements, so a thread's 16 consecutive elements (stride 17) fall in
// distinct banks.
__device__ __forceinline__ int scan_pad(int i) { return i + (i >> 4); }

// fold_nb > 0: partial[] holds the nb = fold_nb raw block sums (no partials
// kernel ran): every block adds those before it itself, in a fixed order, and
// the total of all of them (the same value in every block); block 0 writes it
// to *total_out and adds it to *accum when given.  Only the blocks holding
// elements (those below n, after the n_dev cap) take part; the others exit at
// once.  fold_nb == 0: partial[] holds the scanned prefixes and *total the
// total.
template <typename Tin, typename Tacc, bool kInclusive, bool kNormalize = false>
__global__ void scan_apply(const Tin* __restrict__ in, Tacc* __restrict__ out, int64_t n,
                           const Tacc* __restrict__ partial, const Tacc* __restrict__ total = nullptr,
                           const uint32_t* __restrict__ gather = nullptr, const int64_t* n_dev = nullptr,
                           int64_t fold_nb = 0, Tacc* total_out = nullptr, int64_t* accum = nullptr) {
    __shared__ Tacc tile[kScanTile + kScanTile / 16];
    __shared__ Tacc red[33];
    __shared__ Tacc fold[2];
    pdl_wait();
    pdl_trigger();
    if (n_dev) n = min(n, *n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    Tacc prefix = 0, all = 0;
    if (fold_nb > 0) {
        if (base >= n && blockIdx.x != 0) return;  // uniform per block; block 0 always writes the total
        const int64_t nb_act = min(fold_nb, (n + kScanTile - 1) / kScanTile);
        Tacc a = 0, t = 0;
        for (int64_t i = threadIdx.x; i < nb_act; i += kScanThreads) {
            const Tacc v = partial[i];
            t += v;
            if (i < (int64_t)blockIdx.x) a += v;
        }
        const Tacc ra = block_reduce_sum(a, red);
        if (threadIdx.x == 0) fold[0] = ra;
        __syncthreads();
        const Tacc rt = block_reduce_sum(t, red);
        if (threadIdx.x == 0) fold[1] = rt;
        __syncthreads();
        prefix = fold[0];
        all = fold[1];
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (total_out) *total_out = all;
            if (accum) *accum += (int64_t)all;
        }
    } else {
        if (base < n) prefix = partial[blockIdx.x];
        if (kNormalize) all = *total;
    }
    if (base >= n) return;  // uniform per block
    {
        Tacc v[kScanItems];  // all of the thread's loads in flight before the first store
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            const int i = threadIdx.x + k * kScanThreads;
            const int64_t g = base + i;
            v[k] = g < n ? (Tacc)in[gather ? (int64_t)gather[g] : g] : Tacc(0);
        }
#pragma unroll
        for (int k = 0; k < kScanItems; k++) tile[scan_pad(threadIdx.x + k * kScanThreads)] = v[k];
    }
    __syncthreads();
    Tacc loc[kScanItems];
    Tacc sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        loc[k] = tile[scan_pad(threadIdx.x * kScanItems + k)];
        sum += loc[k];
    }
    Tacc tot;
    Tacc run = block_exclusive_scan(sum, red, &tot) + prefix;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (kInclusive) {
            run += loc[k];
            tile[scan_pad(threadIdx.x * kScanItems + k)] = run;
        } else {
            tile[scan_pad(threadIdx.x * kScanItems + k)] = run;
            run += loc[k];
        }
    }
    __syncthreads();
    if (kNormalize) {
        // One reciprocal per block; the products differ from division by at
        // most one rounding.
        const Tacc rt = Tacc(1) / all;
        for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
            int64_t g = base + i;
            if (g < n) out[g] = (g == n - 1) ? Tacc(1) : tile[scan_pad(i)] * rt;
        }
    } else {
        for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
            int64_t g = base + i;
            if (g < n) out[g] = tile[scan_pad(i)];
        }
    }
}

// Scans of up to kFoldMaxBlocks tiles fold the block sums into the apply
// kernel (each block reads at most that many partials).
constexpr int64_t kFoldMaxBlocks = 2048;

template <typename Tacc>
__global__ void accumulate_total(int64_t* accum, const Tacc* total) {
    pdl_wait();
    *accum += (int64_t)*total;
}

template <typename Tin, typename Tacc, bool kInclusive>
static int scan_impl(const Tin* in, Tacc* out, int64_t n, Tacc* total, void* scratch, cudaStream_t s,
                     int64_t* accum = nullptr) {
    if (n <= 0) {
        if (total) EXAFAC_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(Tacc), s));
        return EXAFAC_OK;
    }
    int64_t nb = ceil_div(n, kScanTile);
    Tacc* partial = reinterpret_cast<Tacc*>(scratch);
    scan_block_sums<Tin, Tacc><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, partial); count_launch();
    if (nb <= kFoldMaxBlocks) {  // each block folds the block sums itself: no partials kernel
        EXAFAC_CUDA_TRY(launch_dependent(scan_apply<Tin, Tacc, kInclusive>, (unsigned)nb, kScanThreads, 0, s, in, out,
                                         n, partial, nullptr, nullptr, nullptr, nb, total, accum));
    } else {
        EXAFAC_CUDA_TRY(launch_dependent(scan_partials_kernel<Tacc>, 1, 1024, 0, s, partial, nb, total));
        count_launch();
        if (accum) {
            EXAFAC_CUDA_TRY(launch_dependent(accumulate_total<Tacc>, 1, 1, 0, s, accum, (const Tacc*)total));
            count_launch();
        }
        EXAFAC_CUDA_TRY(launch_dependent(scan_apply<Tin, Tacc, kInclusive>, (unsigned)nb, kScanThreads, 0, s, in, out,
                                         n, (const Tacc*)partial, nullptr, nullptr, nullptr, 0, nullptr, nullptr));
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total, void* scratch, cudaStream_t s) {
    return scan_impl<int64_t, int64_t, false>(in, out, n, total, scratch, s);
}
int scan_exclusive_u32_to_i64(const uint32_t* in, int64_t* out, int64_t n, int64_t* total, void* scratch,
                              cudaStream_t s, int64_t* accum) {
    return scan_impl<uint32_t, int64_t, false>(in, out, n, total, scratch, s, accum);
}
int scan_inclusive_f64(const double* in, double* out, int64_t n, double* total, void* scratch, cudaStream_t s) {
    return scan_impl<double, double, true>(in, out, n, total, scratch, s);
}
int scan_cdf_f64(const double* in, double* out, int64_t n, double* total, void* scratch, cudaStream_t s,
                 const uint32_t* gather, const int64_t* n_dev) {
    if (n <= 0) return EXAFAC_OK;
    int64_t nb = ceil_div(n, kScanTile);
    double* partial = reinterpret_cast<double*>(scratch);
    scan_block_sums<double, double><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, partial, gather, n_dev);
    count_launch();
    if (nb <= kFoldMaxBlocks) {
        // the grid is sized for the mode; only the blocks below the listed
        // count fold their predecessors' sums
        EXAFAC_CUDA_TRY(launch_dependent(scan_apply<double, double, true, true>, (unsigned)nb, kScanThreads, 0, s, in,
                                         out, n, (const double*)partial, nullptr, gather, n_dev, nb, total, nullptr));
    } else {
        EXAFAC_CUDA_TRY(launch_dependent(scan_partials_kernel<double>, 1, 1024, 0, s, partial, nb, total));
        count_launch();
        EXAFAC_CUDA_TRY(launch_dependent(scan_apply<double, double, true, true>, (unsigned)nb, kScanThreads, 0, s, in,
                                         out, n, (const double*)partial, (const double*)total, gather, n_dev, 0,
                                         nullptr, nullptr));
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;  // 4096
constexpr int kRadixWarps = kRadixThreads / 32;

__device__ __forceinline__ unsigned digit_of(uint64_t lo, uint64_t hi, int shift) {
    uint64_t v;
    if (shift >= 64) v = hi >> (shift - 64);
    else if (shift > 56) v = (lo >> shift) | (hi << (64 - shift));
    else v = lo >> shift;
    return (unsigned)(v & 0xffu);
}

__global__ void radix_hist_kernel(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi, int64_t n,
                                  int shift, uint32_t* __restrict__ hist, int64_t nb) {
    __shared__ uint32_t cnt[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRadixTile;
    for (int i = threadIdx.x; i < kRadixTile; i += blockDim.x) {
        int64_t g = base + i;
        if (g < n) atomicAdd(&cnt[digit_of(lo[g], hi ? hi[g] : 0ull, shift)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(int64_t)d * nb + blockIdx.x] = cnt[d];
}

__global__ void radix_scatter_kernel(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi,
                                     const uint32_t* __restrict__ pay, int64_t n, int shift,
                                     const int64_t* __restrict__ offsets, int64_t nb, uint64_t* __restrict__ lo_out,
                                     uint64_t* __restrict__ hi_out, uint32_t* __restrict__ pay_out) {
    __shared__ uint32_t whist[kRadixWarps][256];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kRadixWarps * 256; i += blockDim.x) (&whist[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRadixTile + (int64_t)w * 32 * kRadixItems;
    unsigned dg[kRadixItems];
    uint32_t rk[kRadixItems];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kRadixItems; r++) {
        int64_t g = base + r * 32 + lane;
        unsigned d = 256;
        if (g < n) d = digit_of(lo[g], hi ? hi[g] : 0ull, shift);
        unsigned mask = __match_any_sync(0xffffffffu, d);
        uint32_t before = (d < 256) ? whist[w][d] : 0u;
        __syncwarp();
        if (d < 256 && (mask & lt) == 0) whist[w][d] = before + __popc(mask);
        __syncwarp();
        dg[r] = d;
        rk[r] = before + __popc(mask & lt);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        uint32_t run = 0;
        for (int ww = 0; ww < kRadixWarps; ww++) {
            uint32_t c = whist[ww][d];
            whist[ww][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRadixItems; r++) {
        int64_t g = base + r * 32 + lane;
        unsigned d = dg[r];
        if (d < 256) {
            int64_t pos = offsets[(int64_t)d * nb + blockIdx.x] + whist[w][d] + rk[r];
            lo_out[pos] = lo[g];
            if (hi) hi_out[pos] = hi[g];
            pay_out[pos] = pay[g];
        }
    }
}

size_t radix_scratch_bytes(int64_t count) {
    int64_t nb = ceil_div(count > 0 ? count : 1, kRadixTile);
    size_t hist = sizeof(uint32_t) * 256 * (size_t)nb;
    size_t offs = sizeof(int64_t) * 256 * (size_t)nb;
    return align_up(hist, 256) + align_up(offs, 256) + align_up(scan_scratch_bytes(256 * nb), 256);
}

int radix_sort_pairs(int64_t count, int bits, int kw, const uint64_t* lo_in, const uint64_t* hi_in,
                     const uint32_t* pay_in, uint64_t* lo_out, uint64_t* hi_out, uint32_t* pay_out, uint64_t* lo_tmp,
                     uint64_t* hi_tmp, uint32_t* pay_tmp, void* scratch, cudaStream_t s) {
    if (count <= 0) return EXAFAC_OK;
    const int64_t nb = ceil_div(count, kRadixTile);
    char* sc = reinterpret_cast<char*>(scratch);
    uint32_t* hist = reinterpret_cast<uint32_t*>(sc);
    int64_t* offs = reinterpret_cast<int64_t*>(sc + align_up(sizeof(uint32_t) * 256 * nb, 256));
    void* scan_sc = sc + align_up(sizeof(uint32_t) * 256 * nb, 256) + align_up(sizeof(int64_t) * 256 * nb, 256);
    const int passes = bits <= 0 ? 0 : (bits + 7) / 8;
    const bool has_hi = kw == 2;
    // Ping-pong so that the last pass writes *_out.
    const uint64_t* src_lo = lo_in;
    const uint64_t* src_hi = hi_in;
    const uint32_t* src_p = pay_in;
    if (passes == 0) {
        EXAFAC_CUDA_TRY(cudaMemcpyAsync(lo_out, lo_in, sizeof(uint64_t) * count, cudaMemcpyDeviceToDevice, s));
        if (has_hi) EXAFAC_CUDA_TRY(cudaMemcpyAsync(hi_out, hi_in, sizeof(uint64_t) * count, cudaMemcpyDeviceToDevice, s));
        EXAFAC_CUDA_TRY(cudaMemcpyAsync(pay_out, pay_in, sizeof(uint32_t) * count, cudaMemcpyDeviceToDevice, s));
        return EXAFAC_OK;
    }
    for (int p = 0; p < passes; p++) {
        const bool last = (p == passes - 1);
        // Destination alternates so the final pass lands in *_out.
        const bool to_out = ((passes - 1 - p) % 2) == 0;
        uint64_t* dlo = to_out ? lo_out : lo_tmp;
        uint64_t* dhi = to_out ? hi_out : hi_tmp;
        uint32_t* dp = to_out ? pay_out : pay_tmp;
        (void)last;
        radix_hist_kernel<<<(unsigned)nb, kRadixThreads, 0, s>>>(src_lo, has_hi ? src_hi : nullptr, count, p * 8, hist,
                                                                 nb); count_launch();
        EXAFAC_CHECK_LAUNCH();
        EXAFAC_TRY(scan_exclusive_u32_to_i64(hist, offs, 256 * nb, nullptr, scan_sc, s));
        radix_scatter_kernel<<<(unsigned)nb, kRadixThreads, 0, s>>>(src_lo, has_hi ? src_hi : nullptr, src_p, count,
                                                                    p * 8, offs, nb, dlo, dhi, dp); count_launch();
        EXAFAC_CHECK_LAUNCH();
        src_lo = dlo;
        src_hi = dhi;
        src_p = dp;
    }
    return EXAFAC_OK;
}

}  // namespace exafac
