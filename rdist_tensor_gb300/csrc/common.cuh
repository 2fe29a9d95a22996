// Shared device/host helpers for the exafac GB300 library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <string>

#include "exafac_gb300.h"

namespace exafac {

constexpr int kMaxModes = 8;
constexpr int kMaxRank = 128;

// Last-error text for the C-ABI (thread-local).
void set_error(const std::string& msg);

// Kernel launches issued by the library since load (exafac_kernel_launches);
// a replayed graph adds the launches it holds.
void count_launch();
void add_launches(long long n);

#define EXAFAC_CUDA_TRY(expr)                                                                     \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            ::exafac::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));              \
            return EXAFAC_ERR_CUDA;                                                               \
        }                                                                                         \
    } while (0)

#define EXAFAC_CHECK_LAUNCH()                                                                     \
    do {                                                                                          \
        cudaError_t _e = cudaGetLastError();                                                      \
        if (_e != cudaSuccess) {                                                                  \
            ::exafac::set_error(std::string("kernel launch: ") + cudaGetErrorString(_e));         \
            return EXAFAC_ERR_CUDA;                                                               \
        }                                                                                         \
    } while (0)

#define EXAFAC_ARG(cond, msg)                                                                     \
    do {                                                                                          \
        if (!(cond)) {                                                                            \
            ::exafac::set_error(msg);                                                             \
            return EXAFAC_ERR_ARG;                                                                \
        }                                                                                         \
    } while (0)

#define EXAFAC_TRY(expr)                                                                          \
    do {                                                                                          \
        int _s = (expr);                                                                          \
        if (_s != EXAFAC_OK) return _s;                                                           \
    } while (0)

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter-based uniforms.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        unsigned lo0 = c.x * 0xD2511F53u, hi0 = __umulhi(c.x, 0xD2511F53u);
        unsigned lo1 = c.z * 0xCD9E8D57u, hi1 = __umulhi(c.z, 0xCD9E8D57u);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Uniform double in [0, 1) from 53 bits of two words.
__device__ __forceinline__ double u53(unsigned a, unsigned b) {
    unsigned long long x = ((unsigned long long)a << 32) | b;
    return (double)(x >> 11) * 0x1.0p-53;
}

// Device error word: kernels that find an out-of-range index record it here
// (first writer wins) and skip the access instead of trapping.
struct DeviceStatus {
    int code;      // EXAFAC_OK or an EXAFAC_ERR_* value
    int where;     // kernel id
    long long a;   // offending value
    long long b;   // bound
};

__device__ __forceinline__ void report(DeviceStatus* st, int code, int where, long long a, long long b) {
    if (st && atomicCAS(&st->code, 0, code) == 0) {
        st->where = where;
        st->a = a;
        st->b = b;
    }
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Bump allocator over a caller-provided device buffer (no cudaMalloc inside
// the library).  In "plan" mode (base == nullptr) it only measures.
struct Arena {
    char* base = nullptr;
    size_t cap = 0;
    size_t used = 0;
    bool overflow = false;
    template <typename T>
    T* take(int64_t count) {
        size_t off = align_up(used, 256);
        size_t bytes = sizeof(T) * (size_t)(count > 0 ? count : 1);
        used = off + bytes;
        if (base == nullptr) return nullptr;
        if (used > cap) {
            overflow = true;
            return nullptr;
        }
        return reinterpret_cast<T*>(base + off);
    }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Number of bits needed to hold coordinates in [0, dim).
inline int bits_for(int64_t dim) {
    int b = 0;
    while (((int64_t)1 << b) < dim) b++;
    return b;
}

// Packed key of the coordinates of all modes except `skip` (most significant
// mode first) — the lexicographic order of SortIdxLookup
// (sort_lookup.hpp:59-69) as an integer order.
struct KeySpec {
    int N;
    int skip;
    int shift[kMaxModes];  // bit offset of mode k's field from the key's LSB (-1: skipped)
    int bits;              // total bits
};

inline KeySpec make_keyspec(int N, const int64_t* dims, int skip) {
    KeySpec s;
    s.N = N;
    s.skip = skip;
    int total = 0;
    for (int k = N - 1; k >= 0; k--) {
        if (k == skip) {
            s.shift[k] = -1;
            continue;
        }
        s.shift[k] = total;
        total += bits_for(dims[k]);
    }
    s.bits = total;
    return s;
}

struct Key128 {
    uint64_t lo, hi;
};

__device__ __forceinline__ Key128 pack_key(const KeySpec& s, const uint32_t* coords) {
    Key128 k{0, 0};
#pragma unroll 1
    for (int m = 0; m < s.N; m++) {
        int sh = s.shift[m];
        if (sh < 0) continue;
        uint64_t c = coords[m];
        if (sh < 64) {
            k.lo |= c << sh;
            if (sh > 32) k.hi |= c >> (64 - sh);
        } else {
            k.hi |= c << (sh - 64);
        }
    }
    return k;
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014)
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}
__device__ __forceinline__ uint64_t hash_key(Key128 k) { return mix64(k.lo ^ mix64(k.hi + 0x9e3779b97f4a7c15ull)); }

}  // namespace exafac
