// Hits of a sampled step grouped by output row (csr_based_spmm's counting
// sort, sort_lookup.hpp:320-346, done as a stable LSD radix sort so that no
// two threads ever update the same counter: Zipf-distributed rows put a large
// share of the hits on a few rows, and atomics on those rows serialise).
//
//   expand     hit h (in sample order) -> key[h] = its output row, plus the
//              sample j and value of the hit (ex_j, ex_val; or, for the
//              mixed forms, one packed 64-bit payload)
//   sort       8-bit digits, per pass: per-tile digit counts (upsweep), a
//              scan of each digit's counts across tiles (spine), a stable
//              scatter of (key, hit index or packed hit) (downsweep)
//   heads      runs of equal keys = touched rows: per-tile run counts, their
//              scan, and the compaction into the touched list and the run
//              starts (seg_start)
//
// The hit count H lives on the device (counters[1]); every kernel reads it
// there and loops over its tiles with a fixed grid, so nothing here waits on
// the host.  Within a row the hits keep sample order, which fixes the order
// of the floating-point sums downstream: results repeat bit for bit.
#include "engine.cuh"

namespace exafac {

constexpr int kHsThreads = 256;
constexpr int kHsItems = 16;
constexpr int kHsTile = kHsThreads * kHsItems;  // 4096 hits per tile
constexpr int kHsWarps = kHsThreads / 32;
constexpr int kHsGrid = 152 * 4;      // upsweep / heads
constexpr int kHsDownGrid = 152 * 2;        // downsweep: one resident wave (99 registers x 256 threads)
constexpr int kHsDownGridPacked = 152 * 3;  // 64-bit payloads, 8 items per thread
constexpr uint32_t kNoItem = 0xffffffffu;

__device__ __forceinline__ int64_t hit_count(const int64_t* counters, int64_t cap) { return min(counters[1], cap); }

__device__ __forceinline__ int64_t owner_in(const int64_t* __restrict__ f_off, int64_t lo, int64_t hi, int64_t h) {
    // last j in [lo, hi) with f_off[j] <= h (f_off[lo] <= h guaranteed)
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (f_off[mid] <= h) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The sample owning the first hit of every expansion chunk (a load-balanced
// search, thread per sample): sample j owns hits [f_off[j], f_off[j] +
// f_len[j]), and the chunk starts c * kExpandChunk in that range are its.
// The samples with hits partition [0, H), so every chunk start has one owner.
__global__ void expand_owner_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                    const int64_t* __restrict__ f_off, const uint32_t* __restrict__ f_len,
                                    uint32_t* __restrict__ first) {
    const int64_t ju = counters[0];
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ju; j += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t len = f_len[j];
        if (len == 0) continue;
        const int64_t a = f_off[j];
        const int64_t b = min(a + (int64_t)len, cap);
        for (int64_t c = (a + kExpandChunk - 1) / kExpandChunk; c * kExpandChunk < b; c++) first[c] = (uint32_t)j;
    }
}

// Hits in sample order: each warp chunk's samples lie between the owners of
// its first hit and of the next chunk's first hit (expand_owner_kernel), and
// each hit's owner is found by a binary search restricted to them.  kPacked
// (mixed forms): the sample and the FP32 value go to one 64-bit payload
// (sample in the low word, value bits in the high word) that travels with
// the key through the sort; otherwise to ex_j / ex_val.
__device__ __forceinline__ uint64_t pack_hit(uint32_t j, float v) {
    return (uint64_t)j | ((uint64_t)__float_as_uint(v) << 32);
}

template <bool kPacked>
__global__ void hit_expand_kernel(const int64_t* __restrict__ counters, int64_t cap, const int64_t* __restrict__ f_off,
                                  const uint32_t* __restrict__ f_start, const uint32_t* __restrict__ first,
                                  const uint32_t* __restrict__ rows_n,
                                  const double* __restrict__ vals_n, uint32_t* __restrict__ key,
                                  uint32_t* __restrict__ ex_j, double* __restrict__ ex_val,
                                  uint64_t* __restrict__ pay64, DeviceStatus* status) {
    const int64_t ju = counters[0];
    int64_t H = counters[1];
    if (H > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) report(status, EXAFAC_ERR_DEVICE, 4, H, cap);
        H = cap;
    }
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c * kExpandChunk < H; c += nwarps) {
        const int64_t h0 = c * kExpandChunk;
        const int64_t h1 = min(H, h0 + kExpandChunk);
        const int64_t jlo = first[c];
        const int64_t jhi = h1 < H ? min((int64_t)first[c + 1] + 1, ju) : ju;
        for (int64_t h = h0 + lane; h < h1; h += 32) {
            const int64_t j = owner_in(f_off, jlo, jhi, h);
            const int64_t p = (int64_t)f_start[j] + (h - f_off[j]);
            key[h] = rows_n[p];
            if (kPacked) {
                pay64[h] = pack_hit((uint32_t)j, narrow_f64(vals_n[p]));
            } else {
                ex_j[h] = (uint32_t)j;
                ex_val[h] = vals_n[p];
            }
        }
    }
}

// Lanes of the warp whose 9-bit value equals this lane's (the warp
// multi-split: one ballot per bit; 256 marks an empty slot).
__device__ __forceinline__ unsigned digit_peers(unsigned d) {
    unsigned m = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < 9; b++) {
        const unsigned bit = (d >> b) & 1u;
        const unsigned bal = __ballot_sync(0xffffffffu, bit);
        m &= bit ? bal : ~bal;
    }
    return m;
}

// Inclusive warp scan.
template <typename T>
__device__ __forceinline__ T warp_inclusive(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block256_exclusive(uint32_t v, uint32_t* wsum) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t inc = warp_inclusive(v);
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    uint32_t pre = 0;
#pragma unroll
    for (int ww = 0; ww < kHsWarps; ww++) pre += (ww < w) ? wsum[ww] : 0u;
    __syncthreads();
    return pre + inc - v;
}

// cnt[d * stride + t] = number of keys in tile t (ITEMS per thread) with digit d.
template <int ITEMS>
__global__ void __launch_bounds__(kHsThreads) hs_upsweep_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                                const uint32_t* __restrict__ keys, int shift,
                                                                uint32_t* __restrict__ cnt, int64_t stride) {
    constexpr int kTile = kHsThreads * ITEMS;
    __shared__ uint32_t c[256];
    const int64_t H = hit_count(counters, cap);
    const int64_t ntiles = (H + kTile - 1) / kTile;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        c[threadIdx.x] = 0;
        __syncthreads();
        const int64_t base = t * kTile;
        unsigned dg[ITEMS];  // all of the thread's loads issued before the first use
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            const int64_t g = base + threadIdx.x + r * kHsThreads;
            dg[r] = g < H ? (keys[g] >> shift) & 255u : 256u;
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            const unsigned d = dg[r];
            const unsigned peers = digit_peers(d);
            if (d < 256 && (peers & lt) == 0) atomicAdd(&c[d], (uint32_t)__popc(peers));
        }
        __syncthreads();
        cnt[(int64_t)threadIdx.x * stride + t] = c[threadIdx.x];
        __syncthreads();
    }
}

// Warp per digit: exclusive scan of the digit's tile counts in place (four
// tiles per lane per round), the digit's total to tot[d].  32 blocks x 8 warps.
template <int ITEMS>
__global__ void hs_spine_kernel(const int64_t* __restrict__ counters, int64_t cap, uint32_t* __restrict__ cnt,
                                int64_t stride, uint32_t* __restrict__ tot) {
    constexpr int kTile = kHsThreads * ITEMS;
    const int64_t H = hit_count(counters, cap);
    const int64_t ntiles = (H + kTile - 1) / kTile;
    const int lane = threadIdx.x & 31;
    const int d = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (d >= 256) return;
    uint32_t* row = cnt + (int64_t)d * stride;
    uint32_t carry = 0;
    for (int64_t b = 0; b < ntiles; b += 128) {
        uint32_t v[4];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t i = b + lane * 4 + k;
            v[k] = i < ntiles ? row[i] : 0u;
            sum += v[k];
        }
        const uint32_t inc = warp_inclusive(sum);
        uint32_t run = carry + inc - sum;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t i = b + lane * 4 + k;
            if (i < ntiles) row[i] = run;
            run += v[k];
        }
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) tot[d] = carry;
}

// Stable scatter of (key, payload) by digit (payload PT: 32-bit hit index
// or 64-bit packed hit).  Items of a tile are taken in
// order warp by warp (warp w owns items [w*32*ITEMS, (w+1)*32*ITEMS) of the
// tile, round r lane l = item w*32*ITEMS + r*32 + l); the multi-split gives each item
// its rank among equal digits of its round, per-warp counters carry the rank
// across rounds, and prefixes over warps and digits give its place in the
// tile's digit order.  The tile is rearranged in shared memory first, so the
// global writes run in contiguous pieces, one per digit.  pin == null: the
// payload is the item's own index (the hit index of the first pass).
template <typename PT, int ITEMS>
__global__ void __launch_bounds__(kHsThreads) hs_downsweep_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                                  const uint32_t* __restrict__ kin,
                                                                  const PT* __restrict__ pin, int shift,
                                                                  const uint32_t* __restrict__ cnt, int64_t stride,
                                                                  const uint32_t* __restrict__ tot,
                                                                  uint32_t* __restrict__ kout,
                                                                  PT* __restrict__ pout) {
    extern __shared__ __align__(16) unsigned char hs_dyn[];  // payloads, then keys, of one tile
    constexpr int kTile = kHsThreads * ITEMS;
    PT* spay = reinterpret_cast<PT*>(hs_dyn);
    uint32_t* skey = reinterpret_cast<uint32_t*>(hs_dyn + sizeof(PT) * kTile);
    __shared__ uint32_t whist[kHsWarps][256];
    __shared__ uint32_t dbase[256];  // digit start in the whole output
    __shared__ uint32_t tstart[256];  // digit start within the tile
    __shared__ uint32_t gbase[256];   // digit start of this tile in the output
    __shared__ uint32_t wsum[kHsWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    dbase[threadIdx.x] = block256_exclusive(tot[threadIdx.x], wsum);
    const int64_t H = hit_count(counters, cap);
    const int64_t ntiles = (H + kTile - 1) / kTile;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
#pragma unroll
        for (int ww = 0; ww < kHsWarps; ww++) whist[ww][threadIdx.x] = 0;
        __syncthreads();
        const int64_t tile0 = t * kTile;
        const int64_t base = tile0 + (int64_t)w * 32 * ITEMS;
        uint32_t kk[ITEMS];
        PT pp[ITEMS];
        uint32_t rk[ITEMS];  // rank among equal digits of the warp; kNoItem for empty slots
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {  // loads first, all in flight together
            const int64_t g = base + r * 32 + lane;
            kk[r] = 0;
            pp[r] = 0;
            rk[r] = kNoItem;
            if (g < H) {
                kk[r] = kin[g];
                pp[r] = pin ? pin[g] : (PT)g;
                rk[r] = 0;
            }
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            const unsigned d = rk[r] == kNoItem ? 256u : (kk[r] >> shift) & 255u;
            const unsigned peers = digit_peers(d);
            const uint32_t before = (d < 256) ? whist[w][d] : 0u;
            __syncwarp();
            if (d < 256 && (peers & lt) == 0) whist[w][d] = before + (uint32_t)__popc(peers);
            __syncwarp();
            rk[r] = (d < 256) ? before + (uint32_t)__popc(peers & lt) : kNoItem;
        }
        __syncthreads();
        {
            const int d = threadIdx.x;
            uint32_t run = 0;
#pragma unroll
            for (int ww = 0; ww < kHsWarps; ww++) {
                const uint32_t c = whist[ww][d];
                whist[ww][d] = run;
                run += c;
            }
            const uint32_t ts = block256_exclusive(run, wsum);
            tstart[d] = ts;
            gbase[d] = dbase[d] + cnt[(int64_t)d * stride + t];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (rk[r] != kNoItem) {
                const unsigned d = (kk[r] >> shift) & 255u;
                const uint32_t l = tstart[d] + whist[w][d] + rk[r];
                skey[l] = kk[r];
                spay[l] = pp[r];
            }
        }
        __syncthreads();
        const int nvalid = (int)min((int64_t)kTile, H - tile0);
        for (int i = threadIdx.x; i < nvalid; i += kHsThreads) {
            const uint32_t k = skey[i];
            const unsigned d = (k >> shift) & 255u;
            const uint32_t dst = gbase[d] + ((uint32_t)i - tstart[d]);
            kout[dst] = k;
            pout[dst] = spay[i];
        }
        __syncthreads();
    }
}

// Run heads (first hit of a row) of the sorted keys, per tile: the tile's
// count, or (compact) the heads themselves written to touched / seg_start at
// the tile's base, and for every chunk of kSegChunkF32 hits the index of the
// run holding its first hit (chunk_seg).  Same item order as the downsweep.
template <bool kCompact>
__global__ void __launch_bounds__(kHsThreads) hs_heads_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                              const uint32_t* __restrict__ keys,
                                                              uint32_t* __restrict__ tile_heads,
                                                              const int64_t* __restrict__ tile_base,
                                                              uint32_t* __restrict__ touched,
                                                              int64_t* __restrict__ seg_start,
                                                              uint32_t* __restrict__ chunk_seg) {
    __shared__ uint32_t wsum[kHsWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t H = hit_count(counters, cap);
    const int64_t ntiles = (H + kHsTile - 1) / kHsTile;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t base = t * kHsTile + (int64_t)w * 32 * kHsItems;
        unsigned heads[kHsItems];
        uint32_t kk[kHsItems];
        uint32_t n = 0;
#pragma unroll
        for (int r = 0; r < kHsItems; r++) {
            const int64_t g = base + r * 32 + lane;
            bool head = false;
            kk[r] = 0;
            if (g < H) {
                kk[r] = keys[g];
                head = (g == 0) || kk[r] != keys[g - 1];
            }
            heads[r] = __ballot_sync(0xffffffffu, head);
            n += (uint32_t)__popc(heads[r]);
        }
        if (lane == 0) wsum[w] = n;
        __syncthreads();
        if (!kCompact) {
            if (threadIdx.x == 0) {
                uint32_t s = 0;
                for (int ww = 0; ww < kHsWarps; ww++) s += wsum[ww];
                tile_heads[t] = s;
            }
        } else {
            int64_t at = tile_base[t];
            for (int ww = 0; ww < w; ww++) at += wsum[ww];
#pragma unroll
            for (int r = 0; r < kHsItems; r++) {
                if ((heads[r] >> lane) & 1u) {
                    const int64_t q = at + __popc(heads[r] & lt);
                    touched[q] = kk[r];
                    seg_start[q] = base + r * 32 + lane;
                }
                // each round is one chunk of kSegChunkF32 hits: the index of
                // the run holding its first hit
                if (lane == 0 && base + r * 32 < H)
                    chunk_seg[(base + r * 32) / kSegChunkF32] = (uint32_t)(at + (heads[r] & 1u) - 1);
                at += __popc(heads[r]);
            }
        }
        __syncthreads();
    }
}

// One block: exclusive scan of the per-tile head counts into tile_base; the
// number of runs T to *touched_count and seg_start[T] = H.  Thread i scans a
// contiguous slice of the tiles.
__global__ void __launch_bounds__(1024) hs_headscan_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                           const uint32_t* __restrict__ tile_heads,
                                                           int64_t* __restrict__ tile_base,
                                                           int64_t* __restrict__ touched_count,
                                                           int64_t* __restrict__ seg_start) {
    __shared__ int64_t wsum[32];
    const int64_t H = hit_count(counters, cap);
    const int64_t ntiles = (H + kHsTile - 1) / kHsTile;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t per = (ntiles + blockDim.x - 1) / blockDim.x;
    const int64_t i0 = min(ntiles, (int64_t)threadIdx.x * per), i1 = min(ntiles, i0 + per);
    int64_t sum = 0;
    for (int64_t i = i0; i < i1; i++) sum += tile_heads[i];
    const int64_t inc = warp_inclusive(sum);
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    int64_t pre = 0, all = 0;
    for (int ww = 0; ww < 32; ww++) {
        pre += (ww < w) ? wsum[ww] : 0;
        all += wsum[ww];
    }
    int64_t run = pre + inc - sum;
    for (int64_t i = i0; i < i1; i++) {
        tile_base[i] = run;
        run += tile_heads[i];
    }
    if (threadIdx.x == 0) {
        *touched_count = all;
        seg_start[all] = H;
    }
}

constexpr int kHsItemsPacked = 8;  // 64-bit payloads: smaller tiles keep 3 blocks per SM resident

size_t hitsort_tile_stride(int64_t nnz) {
    return (size_t)ceil_div(std::max<int64_t>(nnz, 1), kHsThreads * kHsItemsPacked);
}

static int key_bits(int64_t I) {
    int b = 0;
    while (b < 32 && ((int64_t)1 << b) < I) b++;
    return b;
}

// Sorts (hit_key[0], payload) by key: the identity payload (hit index) or
// the packed hits in pay64[0].  Leaves key_sorted / pay_sorted / pay64_sorted.
static int sort_keys(Session& s, int n, bool packed, cudaStream_t st) {
    const int64_t cap = s.nnz;
    const int passes = std::max(1, (key_bits(s.dims[n]) + 7) / 8);
    const int64_t stride = (int64_t)hitsort_tile_stride(s.nnz);
    int src = 0;
    for (int p = 0; p < passes; p++) {
        const int dst = src ^ 1;
        if (packed) {
            constexpr int IT = kHsItemsPacked;
            hs_upsweep_kernel<IT><<<kHsGrid, kHsThreads, 0, st>>>(s.counters, cap, s.hit_key[src], 8 * p, s.hs_cnt,
                                                                 stride);
            count_launch();
            hs_spine_kernel<IT><<<32, 256, 0, st>>>(s.counters, cap, s.hs_cnt, stride, s.hs_tot);
            count_launch();
            const size_t smem = (sizeof(uint64_t) + sizeof(uint32_t)) * kHsThreads * IT;
            hs_downsweep_kernel<uint64_t, IT><<<kHsDownGridPacked, kHsThreads, smem, st>>>(
                s.counters, cap, s.hit_key[src], s.pay64[src], 8 * p, s.hs_cnt, stride, s.hs_tot, s.hit_key[dst],
                s.pay64[dst]);
        } else {
            hs_upsweep_kernel<kHsItems><<<kHsGrid, kHsThreads, 0, st>>>(s.counters, cap, s.hit_key[src], 8 * p,
                                                                       s.hs_cnt, stride);
            count_launch();
            hs_spine_kernel<kHsItems><<<32, 256, 0, st>>>(s.counters, cap, s.hs_cnt, stride, s.hs_tot);
            count_launch();
            const size_t smem = (sizeof(uint32_t) + sizeof(uint32_t)) * kHsTile;
            hs_downsweep_kernel<uint32_t, kHsItems><<<kHsDownGrid, kHsThreads, smem, st>>>(
                s.counters, cap, s.hit_key[src], p == 0 ? nullptr : s.hit_pay[src], 8 * p, s.hs_cnt, stride, s.hs_tot,
                s.hit_key[dst], s.hit_pay[dst]);
        }
        count_launch();
        EXAFAC_CHECK_LAUNCH();
        src = dst;
    }
    s.key_sorted = s.hit_key[src];
    s.pay_sorted = packed ? nullptr : s.hit_pay[src];
    s.pay64_sorted = packed ? s.pay64[src] : nullptr;
    return EXAFAC_OK;
}

int hits_by_row(Session& s, int n, bool packed, cudaStream_t st) {
    const Lookup& L = s.look[n];
    const int64_t cap = s.nnz;
    if (packed && !s.pay64[0]) {
        set_error("packed hits need a session in a mixed precision");
        return EXAFAC_ERR_ARG;
    }
    expand_owner_kernel<<<152 * 4, 256, 0, st>>>(s.counters, cap, s.f_off, s.f_len, s.expand_first);
    count_launch();
    if (packed)
        hit_expand_kernel<true><<<152 * 8, 256, 0, st>>>(s.counters, cap, s.f_off, s.f_start, s.expand_first, L.rows,
                                                         L.vals, s.hit_key[0], nullptr, nullptr, s.pay64[0], s.status);
    else
        hit_expand_kernel<false><<<152 * 8, 256, 0, st>>>(s.counters, cap, s.f_off, s.f_start, s.expand_first,
                                                          L.rows, L.vals, s.hit_key[0], s.ex_j, s.ex_val, nullptr,
                                                          s.status);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    EXAFAC_TRY(sort_keys(s, n, packed, st));
    hs_heads_kernel<false><<<kHsGrid, kHsThreads, 0, st>>>(s.counters, cap, s.key_sorted, s.head_cnt, nullptr,
                                                          nullptr, nullptr, nullptr);
    count_launch();
    hs_headscan_kernel<<<1, 1024, 0, st>>>(s.counters, cap, s.head_cnt, s.head_base, s.counters + 2, s.seg_start);
    count_launch();
    hs_heads_kernel<true><<<kHsGrid, kHsThreads, 0, st>>>(s.counters, cap, s.key_sorted, nullptr, s.head_base,
                                                         s.touched, s.seg_start, s.chunk_seg);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

// Every nonzero as a "hit": key = its mode-n index, payload = its position
// (counters[1] = nnz); used by the exact MTTKRP.
__global__ void nonzero_keys_kernel(int N, int n, int64_t nnz, const uint32_t* __restrict__ idx,
                                    uint32_t* __restrict__ key, int64_t* __restrict__ counters) {
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t0 == 0) counters[1] = nnz;
    for (int64_t i = t0; i < nnz; i += (int64_t)gridDim.x * blockDim.x) key[i] = idx[i * N + n];
}

int nonzeros_by_row(Session& s, int n, cudaStream_t st) {
    nonzero_keys_kernel<<<152 * 8, 256, 0, st>>>(s.N, n, s.nnz, s.idx, s.hit_key[0], s.counters);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return sort_keys(s, n, false, st);
}

}  // namespace exafac
