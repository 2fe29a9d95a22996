// Fit estimate with zero sampling: the reference's legacy
// DistLowRank.compute_estimated_fit (exafac/low_rank_tensor.py:110-184) on
// one GPU.  The squared error over every nonzero is exact; the squared model
// values over the zeros are estimated from Z coordinates drawn uniformly
// over the index space, of which those that are nonzeros of the tensor are
// dropped, and scaled by (prod dims - nnz) / (samples kept):
//
//   fit = 1 - sqrt(sum_nz (x - m)^2 + (prod dims - nnz) mean_kept m(z)^2) / ||X||
//
// The reference found its collisions with a Bloom filter over the nonzeros
// (bloom_filter.cpp:198-252, MurmurHash3), which reports false positives and
// so drops a few true zeros.  Here the membership test is exact: the
// session's mode-0 fibre hash table (the sorted lookup of the sampled
// MTTKRP) gives the fibre of the coordinate's other modes, whose mode-0
// indices are scanned for the coordinate's own.
#include <cmath>

#include "engine.cuh"

namespace exafac {

// m = sum_u sigma_u prod_k U_k[c_k, u] for one coordinate.
__device__ __forceinline__ double model_value(int N, int R, const uint32_t* c, const FactorPtrs& f,
                                              const double* __restrict__ sigma) {
    double value = 0.0;
    for (int u = 0; u < R; u++) {
        double p = sigma[u];
        for (int k = 0; k < N; k++) p *= f.U[k][(int64_t)c[k] * R + u];
        value += p;
    }
    return value;
}

template <typename Slot>
__device__ __forceinline__ bool slot_is(const Slot& sl, Key128 k);
template <>
__device__ __forceinline__ bool slot_is<Slot1>(const Slot1& sl, Key128 k) {
    return sl.key == k.lo;
}
template <>
__device__ __forceinline__ bool slot_is<Slot2>(const Slot2& sl, Key128 k) {
    return sl.lo == k.lo && sl.hi == k.hi;
}

// Is coordinate c a nonzero?  Probe the mode-0 fibre table (bounded as the
// lookup kernel's), then scan the fibre's mode-0 indices.
template <typename Slot>
__device__ __forceinline__ bool is_nonzero(const KeySpec& spec, const Slot* __restrict__ slots, int64_t mask,
                                           const uint32_t* __restrict__ rows0, const uint32_t* c) {
    const Key128 key = pack_key(spec, c);
    int64_t h = (int64_t)(hash_key(key) & (uint64_t)mask);
    for (int64_t probe = 0; probe <= mask; probe++) {
        const Slot sl = slots[h];
        if (sl.start == kEmpty) return false;
        if (slot_is(sl, key)) {
            for (uint32_t p = 0; p < sl.len; p++)
                if (rows0[sl.start + p] == c[0]) return true;
            return false;
        }
        h = (h + 1) & mask;
    }
    return false;
}

constexpr int kEstBlocks = 152 * 8;

// Block partials (fixed order) of sum over nonzeros of (x - m)^2.
__global__ void nonzero_loss_kernel(int N, int R, int64_t nnz, const uint32_t* __restrict__ idx,
                                    const double* __restrict__ vals, FactorPtrs f, const double* __restrict__ sigma,
                                    double* __restrict__ part) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = vals[i] - model_value(N, R, idx + i * N, f, sigma);
        acc = fma(d, d, acc);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Block partials of sum over kept zero samples of m(z)^2 and of the kept
// count.  Coordinates from zidx (Z x N) or, when null, from Philox4x32-10
// keyed by seed: sample t uses counter (t, 0, 0, 0); coordinate k is
// floor(u_k dims[k]) with u_k a 32-bit uniform (k < 4: word k of the block;
// k >= 4: word k - 4 of the block at counter (t, 1, 0, 0)).
template <typename Slot>
__global__ void zero_loss_kernel(int N, int R, int64_t Z, const uint32_t* __restrict__ zidx, uint64_t seed,
                                 const int64_t* __restrict__ dims, KeySpec spec, const Slot* __restrict__ slots,
                                 int64_t mask, const uint32_t* __restrict__ rows0, FactorPtrs f,
                                 const double* __restrict__ sigma, double* __restrict__ part,
                                 unsigned long long* __restrict__ kept_part) {
    __shared__ double red[256];
    __shared__ unsigned long long cnt[256];
    double acc = 0.0;
    unsigned long long kept = 0;
    const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < Z; t += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c[kMaxModes];
        if (zidx) {
            for (int k = 0; k < N; k++) c[k] = zidx[t * N + k];
        } else {
            const uint4 r0 = philox4x32_10(make_uint4((unsigned)t, (unsigned)(t >> 32), 0u, 0u), key);
            const uint4 r1 = N > 4 ? philox4x32_10(make_uint4((unsigned)t, (unsigned)(t >> 32), 1u, 0u), key)
                                   : make_uint4(0u, 0u, 0u, 0u);
            const unsigned w[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            for (int k = 0; k < N; k++) c[k] = (uint32_t)(((uint64_t)w[k] * (uint64_t)dims[k]) >> 32);
        }
        if (is_nonzero(spec, slots, mask, rows0, c)) continue;
        const double m = model_value(N, R, c, f, sigma);
        acc = fma(m, m, acc);
        kept++;
    }
    red[threadIdx.x] = acc;
    cnt[threadIdx.x] = kept;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
            cnt[threadIdx.x] += cnt[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = red[0];
        kept_part[blockIdx.x] = cnt[0];
    }
}

// out[0] = sum of part[0..n), out[1] = sum of part[n..2n) (as double), out[2]
// = sum of the kept counts: one thread, in order.
__global__ void estfit_finish_kernel(int n, const double* __restrict__ part, const unsigned long long* __restrict__ kp,
                                     double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    unsigned long long k = 0;
    for (int i = 0; i < n; i++) a += part[i];
    for (int i = 0; i < n; i++) b += part[n + i];
    for (int i = 0; i < n; i++) k += kp[i];
    out[0] = a;
    out[1] = b;
    out[2] = (double)k;
}

int estimated_fit(Session& s, int64_t Z, const uint32_t* zero_idx, uint64_t seed, double* fit,
                              int64_t* kept, cudaStream_t st) {
    EXAFAC_ARG(Z >= 1, "exafac_als_estimated_fit: the zero sample count must be >= 1");
    EXAFAC_ARG(fit != nullptr, "exafac_als_estimated_fit: null fit");
    FactorPtrs f;
    for (int k = 0; k < kMaxModes; k++) f.U[k] = k < s.N ? s.F.U[k] : nullptr;
    double* part = s.fitpart;  // 2 x kEstBlocks doubles
    unsigned long long* kp = reinterpret_cast<unsigned long long*>(s.part);  // the Gram partials are idle here
    nonzero_loss_kernel<<<kEstBlocks, 256, 0, st>>>(s.N, s.R, s.nnz, s.idx, s.vals, f, s.F.sigma, part);
    count_launch();
    const Lookup& L = s.look[0];
    if (L.kw == 1)
        zero_loss_kernel<Slot1><<<kEstBlocks, 256, 0, st>>>(s.N, s.R, Z, zero_idx, seed, s.dims_dev, L.spec,
                                                            (const Slot1*)L.slots, L.nslots - 1, L.rows, f, s.F.sigma,
                                                            part + kEstBlocks, kp);
    else
        zero_loss_kernel<Slot2><<<kEstBlocks, 256, 0, st>>>(s.N, s.R, Z, zero_idx, seed, s.dims_dev, L.spec,
                                                            (const Slot2*)L.slots, L.nslots - 1, L.rows, f, s.F.sigma,
                                                            part + kEstBlocks, kp);
    count_launch();
    estfit_finish_kernel<<<1, 32, 0, st>>>(kEstBlocks, part, kp, s.scal + 3);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    double v[3];
    EXAFAC_CUDA_TRY(cudaMemcpyAsync(v, s.scal + 3, sizeof(v), cudaMemcpyDeviceToHost, st));
    EXAFAC_CUDA_TRY(cudaStreamSynchronize(st));
    double dense = 1.0;
    for (int k = 0; k < s.N; k++) dense *= (double)s.dims[k];
    const double zeros = dense - (double)s.nnz;
    const double zero_loss = v[2] > 0 ? v[1] * zeros / v[2] : 0.0;
    *fit = 1.0 - std::sqrt(v[0] + zero_loss) / s.tensor_norm;
    if (kept) *kept = (int64_t)v[2];
    return EXAFAC_OK;
}

}  // namespace exafac
