// Hits of a sampled step grouped by output row (csr_based_spmm's counting
// sort, sort_lookup.hpp:320-346, done as a stable LSD radix sort so that no
// two threads ever update the same counter: Zipf-distributed rows put a large
// share of the hits on a few rows, and atomics on those rows serialise).
//
//   expand     hit h (in sample order) -> key[h] = its output row, plus the
//              sample j and value of the hit (ex_j, ex_val; or, for the
//              mixed forms, one packed 64-bit payload)
//   sort       8-bit digits, LSD.  One read of the keys counts every pass's
//              digits (os_hist); then one kernel per pass (os_downsweep) ranks
//              a tile, publishes its digit counts and resolves the counts of
//              the tiles before it by a decoupled look-back (Merrill and
//              Garland's single-pass scan, as in Adinets and Merrill's
//              Onesweep), and scatters (key, hit index or packed hit) stably
//   runs       runs of equal keys = touched rows, in one pass (hs_runs):
//              each tile counts its run heads, takes the count of the heads
//              before it by the same kind of look-back, and writes its heads
//              to the touched list and the run starts (seg_start)
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
constexpr int kHsGrid = 152 * 4;      // heads
constexpr int kHsDownGrid = 152 * 2;        // downsweep: one resident wave (256 threads)
constexpr int kHsDownGridPacked = 152 * 2;  // 64-bit payloads, 16 items per thread
constexpr int kHistGrid = 152 * 2;          // os_hist
constexpr uint32_t kStatAgg = 1u << 30;     // look-back status: the tile's own count
constexpr uint32_t kStatPrefix = 2u << 30;  // look-back status: the inclusive prefix
constexpr uint32_t kStatValue = (1u << 30) - 1;
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
    pdl_wait();
    pdl_trigger();
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
    pdl_wait();
    pdl_trigger();
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

// Lanes of the warp whose digit equals this lane's (the warp multi-split;
// 256 marks an empty slot): one match instruction.
__device__ __forceinline__ unsigned digit_peers(unsigned d) { return __match_any_sync(0xffffffffu, d); }

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

// Digit counts of every pass in one read of the keys: hist[p * 256 + d] =
// number of keys whose digit p is d (hist zeroed beforehand).  Each warp
// counts its items by multi-split (one shared-memory add per distinct digit
// of a round), each block adds its histograms once (aux cleared beforehand:
// the passes' tile counters aux[0..3] and the histograms aux[4..]).  Block 0
// also advances the look-back epoch (counters[kSortEpochSlot] += 5): every
// pass of this sort marks its status words with a fresh epoch, so the status
// array is never cleared.
__global__ void __launch_bounds__(kHsThreads) os_hist_kernel(int64_t* __restrict__ counters, int64_t cap,
                                                             const uint32_t* __restrict__ keys, int passes,
                                                             uint32_t* __restrict__ aux) {
    constexpr int kItems = 16;
    constexpr int kTile = kHsThreads * kItems;
    // per-warp histograms, so hot digits contend only within a warp
    pdl_trigger();
    __shared__ uint32_t h[kHsWarps][4][256];
    for (int e = threadIdx.x; e < kHsWarps * 4 * 256; e += blockDim.x) (&h[0][0][0])[e] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) counters[kSortEpochSlot] += 5;
    __syncthreads();
    const int64_t H = hit_count(counters, cap);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int64_t base = (int64_t)blockIdx.x * kTile; base < H; base += (int64_t)gridDim.x * kTile) {
        uint32_t k[kItems];  // all of the thread's loads in flight before the first use
        bool on[kItems];
#pragma unroll
        for (int r = 0; r < kItems; r++) {
            const int64_t g = base + r * kHsThreads + threadIdx.x;
            on[r] = g < H;
            k[r] = on[r] ? keys[g] : 0u;
        }
        for (int p = 0; p < passes; p++) {
            uint32_t* hw = h[w][p];
#pragma unroll
            for (int r = 0; r < kItems; r++) {
                const unsigned d = on[r] ? (k[r] >> (8 * p)) & 255u : 256u;
                // a digit shared by the whole warp (the high digits of
                // Zipf-distributed rows) is one add; otherwise one shared
                // atomic per item
                const unsigned d0 = __shfl_sync(0xffffffffu, d, 0);
                if (__all_sync(0xffffffffu, d == d0)) {
                    if (lane == 0 && d0 < 256) hw[d0] += 32u;
                } else if (d < 256) {
                    atomicAdd(&hw[d], 1u);
                }
            }
            __syncwarp();
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < passes * 256; e += blockDim.x) {
        uint32_t v = 0;
#pragma unroll
        for (int ww = 0; ww < kHsWarps; ww++) v += (&h[ww][0][0])[e];
        if (v) atomicAdd(&aux[4 + e], v);
    }
}

// One pass: stable scatter of (key, payload) by digit (payload PT: 32-bit hit
// index or 64-bit packed hit).  Blocks take tiles in order from a counter, so
// a tile's predecessors are always held by running blocks.  Items of a tile
// are taken warp by warp (warp w owns items [w*32*ITEMS, (w+1)*32*ITEMS) of
// the tile, round r lane l = item w*32*ITEMS + r*32 + l); the multi-split
// gives each item its rank among equal digits of its round, per-warp counters
// carry the rank across rounds, and prefixes over warps and digits give its
// place in the tile's digit order.  Thread d then publishes the tile's count
// of digit d (status = epoch | kStatAgg | count), sums the counts of earlier
// tiles back to the first inclusive prefix it meets, and publishes its own
// inclusive prefix.  The tile is rearranged in shared memory first, so the
// global writes run in contiguous pieces, one per digit.  pin == null: the
// payload is the item's own index (the hit index of the first pass).  A
// look-back wait that outlasts kSpinLimit polls records an error and counts
// as a zero prefix (the output is then invalid, and reported).
__device__ __forceinline__ uint64_t os_load(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void os_store(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <typename PT, int ITEMS>
__global__ void __launch_bounds__(kHsThreads) os_downsweep_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                                  const uint32_t* __restrict__ kin,
                                                                  const PT* __restrict__ pin, int pass,
                                                                  uint32_t* __restrict__ aux,
                                                                  uint64_t* __restrict__ status,
                                                                  uint32_t* __restrict__ kout,
                                                                  PT* __restrict__ pout, DeviceStatus* err,
                                                                  uint32_t spin_limit, int64_t withhold) {
    extern __shared__ __align__(16) unsigned char hs_dyn[];  // payloads, then keys, of one tile
    constexpr int kTile = kHsThreads * ITEMS;
    PT* spay = reinterpret_cast<PT*>(hs_dyn);
    uint32_t* skey = reinterpret_cast<uint32_t*>(hs_dyn + sizeof(PT) * kTile);
    __shared__ uint32_t whist[kHsWarps][256];
    __shared__ uint32_t dbase[256];   // digit start in the whole output
    __shared__ uint32_t tstart[256];  // digit start within the tile
    __shared__ uint32_t gbase[256];   // digit start of this tile in the output
    __shared__ uint32_t wsum[kHsWarps];
    __shared__ int64_t tile_sh;
    pdl_wait();
    pdl_trigger();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int shift = 8 * pass;
    const uint64_t epoch = (uint64_t)(uint32_t)(counters[kSortEpochSlot] + pass) << 32;
    dbase[threadIdx.x] = block256_exclusive(aux[4 + pass * 256 + threadIdx.x], wsum);
    const int64_t H = hit_count(counters, cap);
    const int64_t ntiles = (H + kTile - 1) / kTile;
    for (;;) {
        if (threadIdx.x == 0) tile_sh = (int64_t)atomicAdd(&aux[pass], 1u);
#pragma unroll
        for (int ww = 0; ww < kHsWarps; ww++) whist[ww][threadIdx.x] = 0;
        __syncthreads();
        const int64_t t = tile_sh;
        if (t >= ntiles) break;  // uniform
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
            // publish this tile's count, then look back for the prefix
            uint64_t* my = status + t * 256 + d;
            uint32_t excl = 0;
            const bool publish = t != withhold;  // withhold >= 0 only under the wait-limit test hook
            if (t == 0) {
                if (publish) os_store(my, epoch | kStatPrefix | run);
            } else {
                if (publish) os_store(my, epoch | kStatAgg | run);
                // windows of kLook predecessors: their status words are loaded
                // together, then taken in order back to the first prefix
                constexpr int kLook = 4;
                bool done = false;
                for (int64_t top = t - 1; top >= 0 && !done; top -= kLook) {
                    uint64_t v[kLook];
#pragma unroll
                    for (int q = 0; q < kLook; q++) v[q] = top - q >= 0 ? os_load(status + (top - q) * 256 + d) : 0;
#pragma unroll
                    for (int q = 0; q < kLook; q++) {
                        if (done || top - q < 0) continue;
                        const uint64_t* src = status + (top - q) * 256 + d;
                        uint64_t x = v[q];
                        for (uint32_t it = 0; (x & 0xffffffff00000000ull) != epoch; it++) {
                            // give up after spin_limit polls, or at once when another wait already did
                            if (it >= spin_limit || ((it & 1023u) == 1023u && *(volatile int*)&err->code != 0)) {
                                report(err, EXAFAC_ERR_TIMEOUT, 9, top - q, t);
                                x = epoch | kStatPrefix;
                                break;
                            }
                            if (it >= 32) __nanosleep(64);
                            x = os_load(src);
                        }
                        excl += (uint32_t)x & kStatValue;
                        done = ((uint32_t)x & kStatPrefix) != 0;
                    }
                }
                if (publish) os_store(my, epoch | kStatPrefix | (excl + run));
            }
            const uint32_t ts = block256_exclusive(run, wsum);
            tstart[d] = ts;
            gbase[d] = dbase[d] + excl;
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
            if (dst < (uint64_t)H) {  // always, unless a failed look-back (reported) broke the prefixes
                kout[dst] = k;
                pout[dst] = spay[i];
            }
        }
        __syncthreads();
    }
}

// Runs of equal rows in the sorted keys, in one pass: each tile of kHsTile
// hits (claimed in order through aux[kRunsTileSlot]) counts its run heads
// (first hit of a row), publishes the count in its status word (slot 0 of
// its status row, under the sort's epoch + 4: the digit passes use + 0..3)
// and takes its exclusive prefix from a block-wide look-back over earlier
// tiles (kHsThreads of them per window, one per thread), which have all been
// claimed by running blocks and publish their counts before they look back
// themselves.  It then writes its heads to
// touched / seg_start at that prefix, marks their rows in the step's row
// bitmap (rowbits, cleared beforehand) and, for every chunk of kSegChunkF32
// hits, records the index of the run holding its first hit (chunk_seg).  The
// last tile writes the number of runs T to *touched_count and seg_start[T] =
// H.  A look-back wait that outlasts kSpinLimit polls records an error and
// counts as a zero prefix (the output is then invalid, and reported).
constexpr int kRunsTileSlot = 4 + 4 * 256;  // in os_aux, after the sort's tile counters and histograms

__global__ void __launch_bounds__(kHsThreads) hs_runs_kernel(const int64_t* __restrict__ counters, int64_t cap,
                                                             const uint32_t* __restrict__ keys,
                                                             uint32_t* __restrict__ aux, uint64_t* __restrict__ status,
                                                             uint32_t* __restrict__ touched,
                                                             int64_t* __restrict__ seg_start,
                                                             uint32_t* __restrict__ chunk_seg,
                                                             uint32_t* __restrict__ rowbits,
                                                             int64_t* __restrict__ touched_count, DeviceStatus* err,
                                                             uint32_t spin_limit) {
    __shared__ uint32_t wsum[kHsWarps];
    __shared__ int64_t tile_sh;
    __shared__ int first_sh;
    __shared__ uint32_t red[kHsWarps];
    pdl_wait();
    pdl_trigger();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // A digit pass whose look-back ran out (reported) leaves an unsorted key
    // array whose unwritten positions hold stale rows, possibly of another
    // mode: the step then has no runs, so no later kernel indexes by them.
    const bool sort_failed = *(volatile int*)&err->code == EXAFAC_ERR_TIMEOUT;
    const int64_t H = sort_failed ? 0 : hit_count(counters, cap);
    // and the kernels after this one see no hits either (every block has read
    // the count above through sort_failed, not from counters[1])
    if (sort_failed && blockIdx.x == 0 && threadIdx.x == 0) const_cast<int64_t*>(counters)[1] = 0;
    const int64_t ntiles = (H + kHsTile - 1) / kHsTile;
    const uint64_t epoch = (uint64_t)(uint32_t)(counters[kSortEpochSlot] + 4) << 32;
    if (ntiles == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *touched_count = 0;
            seg_start[0] = 0;
        }
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) tile_sh = (int64_t)atomicAdd(&aux[kRunsTileSlot], 1u);
        __syncthreads();
        const int64_t t = tile_sh;
        if (t >= ntiles) break;  // uniform
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
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kHsWarps; ww++) run += wsum[ww];
        uint64_t* my = status + t * 256;
        uint32_t excl = 0;  // the same in every thread: block-wide sums of the same words
        if (t == 0) {
            if (threadIdx.x == 0) os_store(my, epoch | kStatPrefix | run);
        } else {
            if (threadIdx.x == 0) os_store(my, epoch | kStatAgg | run);
            // windows of kHsThreads predecessors, thread i on tile top - i
            for (int64_t top = t - 1; top >= 0; top -= kHsThreads) {
                const int64_t src_t = top - threadIdx.x;
                uint64_t x = epoch | kStatAgg;  // threads past tile 0 hold a zero count
                if (src_t >= 0) {
                    const uint64_t* src = status + src_t * 256;
                    x = os_load(src);
                    for (uint32_t it = 0; (x & 0xffffffff00000000ull) != epoch; it++) {
                        // give up after spin_limit polls, or at once when another wait already did
                        if (it >= spin_limit || ((it & 1023u) == 1023u && *(volatile int*)&err->code != 0)) {
                            report(err, EXAFAC_ERR_TIMEOUT, 12, src_t, t);
                            x = epoch | kStatPrefix;
                            break;
                        }
                        if (it >= 32) __nanosleep(64);
                        x = os_load(src);
                    }
                }
                // the nearest prefix (lowest thread) ends the look-back: threads up to it count
                if (threadIdx.x == 0) first_sh = kHsThreads;
                __syncthreads();
                if (((uint32_t)x & kStatPrefix) != 0) atomicMin(&first_sh, (int)threadIdx.x);
                __syncthreads();
                const int first = first_sh;
                uint32_t v = (int)threadIdx.x <= first ? ((uint32_t)x & kStatValue) : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0) red[w] = v;
                __syncthreads();
#pragma unroll
                for (int ww = 0; ww < kHsWarps; ww++) excl += red[ww];
                __syncthreads();  // red and first_sh are rewritten by the next window
                if (first < kHsThreads) break;  // uniform
            }
            if (threadIdx.x == 0) os_store(my, epoch | kStatPrefix | (excl + run));
        }
        if (threadIdx.x == 0 && t == ntiles - 1) {
            *touched_count = (int64_t)excl + run;
            seg_start[(int64_t)excl + run] = H;
        }
        int64_t at = excl;
        for (int ww = 0; ww < w; ww++) at += wsum[ww];
#pragma unroll
        for (int r = 0; r < kHsItems; r++) {
            const bool hd = (heads[r] >> lane) & 1u;
            if (hd) {
                const int64_t q = at + __popc(heads[r] & lt);
                touched[q] = kk[r];
                seg_start[q] = base + r * 32 + lane;
            }
            {  // the step's row bitmap: the round's rows are sorted, so equal
                // 32-row words are runs of lanes; a segmented OR-scan leaves each
                // run's bits in its last lane, which makes the one atomic
                const unsigned word = kk[r] >> 5;
                unsigned bits = hd ? 1u << (kk[r] & 31) : 0u;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned b = __shfl_up_sync(0xffffffffu, bits, o);
                    const unsigned wo = __shfl_up_sync(0xffffffffu, word, o);
                    if (lane >= o && wo == word) bits |= b;
                }
                const unsigned wn = __shfl_down_sync(0xffffffffu, word, 1);
                if (bits && (lane == 31 || wn != word)) atomicOr(&rowbits[word], bits);
            }
            // a round that starts a chunk of kSegChunkF32 hits: the index
            // of the run holding its first hit
            if (lane == 0 && base + r * 32 < H && (base + r * 32) % kSegChunkF32 == 0)
                chunk_seg[(base + r * 32) / kSegChunkF32] = (uint32_t)(at + (heads[r] & 1u) - 1);
            at += __popc(heads[r]);
        }
        __syncthreads();
    }
}

constexpr int kHsItemsPacked = 16;  // 64-bit payloads: 4096-hit tiles, 2 blocks per SM

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
    if (cap >= ((int64_t)1 << 30)) {
        set_error("the row sort holds hit counts in 30 bits: at most 2^30 - 1 nonzeros");
        return EXAFAC_ERR_ARG;
    }
    const int passes = std::max(1, (key_bits(s.dims[n]) + 7) / 8);
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.os_aux, 0, sizeof(uint32_t) * (kRunsTileSlot + 1), st));
    os_hist_kernel<<<kHistGrid, kHsThreads, 0, st>>>(s.counters, cap, s.hit_key[0], passes, s.os_aux);
    count_launch();
    int src = 0;
    for (int p = 0; p < passes; p++) {
        const int dst = src ^ 1;
        if (packed) {
            constexpr int IT = kHsItemsPacked;
            const size_t smem = (sizeof(uint64_t) + sizeof(uint32_t)) * kHsThreads * IT;
            EXAFAC_CUDA_TRY(cudaFuncSetAttribute(os_downsweep_kernel<uint64_t, IT>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            EXAFAC_CUDA_TRY(launch_dependent(os_downsweep_kernel<uint64_t, IT>, kHsDownGridPacked, kHsThreads, smem, st,
                                             s.counters, cap, s.hit_key[src], s.pay64[src], p, s.os_aux, s.os_status,
                                             s.hit_key[dst], s.pay64[dst], s.status, s.wait_polls,
                                             p == 0 ? s.withhold_tile : (int64_t)-1));
        } else {
            const size_t smem = (sizeof(uint32_t) + sizeof(uint32_t)) * kHsTile;
            EXAFAC_CUDA_TRY(launch_dependent(os_downsweep_kernel<uint32_t, kHsItems>, kHsDownGrid, kHsThreads, smem, st,
                                             s.counters, cap, s.hit_key[src], p == 0 ? nullptr : s.hit_pay[src], p,
                                             s.os_aux, s.os_status, s.hit_key[dst], s.hit_pay[dst], s.status,
                                             s.wait_polls, p == 0 ? s.withhold_tile : (int64_t)-1));
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
    EXAFAC_CUDA_TRY(cudaMemsetAsync(s.rowbits, 0, sizeof(uint32_t) * ceil_div(s.dims[n], 32), st));
    expand_owner_kernel<<<152 * 4, 256, 0, st>>>(s.counters, cap, s.f_off, s.f_len, s.expand_first);
    count_launch();
    if (packed)
        EXAFAC_CUDA_TRY(launch_dependent(hit_expand_kernel<true>, 152 * 8, 256, 0, st, s.counters, cap, s.f_off,
                                         s.f_start, s.expand_first, L.rows, L.vals, s.hit_key[0], nullptr, nullptr,
                                         s.pay64[0], s.status));
    else
        EXAFAC_CUDA_TRY(launch_dependent(hit_expand_kernel<false>, 152 * 8, 256, 0, st, s.counters, cap, s.f_off,
                                         s.f_start, s.expand_first, L.rows, L.vals, s.hit_key[0], s.ex_j, s.ex_val,
                                         nullptr, s.status));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    EXAFAC_TRY(sort_keys(s, n, packed, st));
    EXAFAC_CUDA_TRY(launch_dependent(hs_runs_kernel, kHsGrid, kHsThreads, 0, st, s.counters, cap, s.key_sorted,
                                     s.os_aux, s.os_status, s.touched, s.seg_start, s.chunk_seg, s.rowbits,
                                     s.counters + 2, s.status, s.wait_polls));
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
