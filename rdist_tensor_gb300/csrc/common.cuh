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

// Polls of a device-side wait (a look-back status word, an MMA barrier)
// before the wait is declared failed (EXAFAC_ERR_TIMEOUT).
constexpr uint32_t kSpinLimit = 1u << 22;

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

// Conversions between binary32 and binary64 in integer arithmetic.  GB300
// retires about two FP64 operations (conversions included) per clock per SM
// against ~116 FP32 ones, so a hardware conversion per element costs more than
// all the FP32 arithmetic around it.  Both follow IEEE 754 directly: the two
// formats differ in exponent bias (127 / 1023) and mantissa width (23 / 52).
//
// widen_f32: exact.  A normal value keeps sign and mantissa and moves its
// exponent by 1023 - 127 = 896; a subnormal one (mag x 2^-149) is normalised
// by its leading bit; infinities and NaNs keep their mantissa bits.
__device__ __forceinline__ double widen_f32(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t mag = b & 0x7fffffffu;
    const uint32_t sign = b & 0x80000000u;
    uint32_t hi = sign | ((mag >> 3) + (896u << 20)), lo = mag << 29;
    if (__builtin_expect(mag - 0x00800000u >= 0x7f000000u, 0)) {
        if (mag == 0) {
            hi = sign;
        } else if (mag >= 0x7f800000u) {
            hi = sign | 0x7ff00000u | ((mag >> 3) & 0x000fffffu);
        } else {  // subnormal: leading bit k in [0, 22], value 1.f x 2^(k - 149)
            const int k = 31 - __clz(mag);
            const uint64_t m = ((uint64_t)mag << (52 - k)) & 0x000fffffffffffffull;
            hi = sign | ((uint32_t)(k + 874) << 20) | (uint32_t)(m >> 32);
            lo = (uint32_t)m;
        }
    }
    return __hiloint2double((int)hi, (int)lo);
}

// narrow_f64: round to nearest, ties to even, as the ordinary conversion.
// The 53-bit significand is cut to 24 bits (normal results) or to the
// subnormal grid of 2^-149; a carry out of the mantissa moves the exponent
// up (to infinity past the largest float).
__device__ __forceinline__ float narrow_f64(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t mhi = hi & 0x7fffffffu;
    const uint32_t e = mhi >> 20;
    if (__builtin_expect(e - 897u < 254u, 1)) {  // normal float range before rounding
        const uint32_t keep = ((mhi - (896u << 20)) << 3) | (lo >> 29);
        const uint32_t rem = lo & 0x1fffffffu;
        const uint32_t up = (rem > 0x10000000u) | ((rem == 0x10000000u) & keep);
        return __uint_as_float(sign | (keep + up));
    }
    if (e == 2047u) return __uint_as_float(((mhi & 0x000fffffu) | lo) == 0 ? (sign | 0x7f800000u) : (sign | 0x7fffffffu));
    if (e >= 1151u) return __uint_as_float(sign | 0x7f800000u);  // beyond the float range
    if (e < 873u) return __uint_as_float(sign);                    // below half the least subnormal
    // subnormal result: significand M (53 bits) x 2^(e - 1075) on the grid 2^-149
    const uint64_t M = ((uint64_t)((mhi & 0x000fffffu) | 0x00100000u) << 32) | lo;
    const uint32_t s = 926u - e;  // 30 .. 53
    const uint64_t q = M >> s, rem = M & ((1ull << s) - 1), half = 1ull << (s - 1);
    const uint64_t up = (rem > half) | ((rem == half) & q);
    return __uint_as_float(sign | (uint32_t)(q + up));
}

// Compensated FP32 accumulation (Knuth's TwoSum: hi + lo carries the running
// sum to about twice FP32 precision), for sums over many tiles kept off the
// FP64 pipe.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float xp = s - hi;
    const float hp = s - xp;
    lo += (hi - hp) + (x - xp);
    hi = s;
}

// Programmatic dependent launch.  A kernel launched by launch_dependent()
// may be scheduled while the kernel before it in the stream is finishing; it
// calls pdl_wait() before anything else, which returns once that kernel has
// completed and its writes are visible.  pdl_trigger() lets the next such
// kernel be scheduled as soon as every block of this one has started.  Both
// are no-ops for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// dependent = false gives an ordinary launch (for a launch whose stream
// predecessor is not always a kernel).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent_if(bool dependent, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                       cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = dependent ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args... args) {
    return launch_dependent_if(true, kernel, grid, block, smem, st, args...);
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
