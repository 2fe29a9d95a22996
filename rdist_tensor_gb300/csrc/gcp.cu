// Generalized CP on sampled entries: the model at sampled coordinates, its
// adjoint (the sampled MTTKRP of the loss derivatives into every factor),
// and a stratified entry sampler.  No counterpart in the reference, whose
// nearest relatives are execute_exact_mttkrp (sort_lookup.hpp:440-495) and
// the zero-sampling fit estimate of exafac/low_rank_tensor.py:110-184.
//
//   model     m_j = sum_r prod_k U_k[i_jk, r]                 warp per entry
//   adjoint   G_n[i_jn, :] += g_j * prod_{k != n} U_k[i_jk, :]  warp per entry,
//             every mode from one load of the entry's N factor rows; the
//             Khatri-Rao rows are recomputed here, never stored
//   sampler   J_nz nonzeros uniformly (weight nnz / J_nz) and J_z coordinates
//             uniformly (value 0, weight (prod dims - nnz) / J_z), Philox
//   adam      one Adam step over all factors in one launch, fused with the
//             projection onto nonnegative factors: 7 words of traffic per
//             parameter (parameter, moments read and written; gradient read)
//
// The adjoint accumulates with atomic adds, so its last bits depend on the
// order in which entries that share a row arrive.
#include <cmath>
#include <type_traits>

#include "common.cuh"

namespace exafac {

template <typename T>
struct PtrsT {
    T* p[kMaxModes];
};

struct Dims {
    int64_t d[kMaxModes];
};

// Loads the entry's coordinates (lane k holds mode k) and checks them against
// the mode sizes; an entry with an out-of-range coordinate is skipped and
// flagged in *status (when given).
__device__ __forceinline__ bool load_entry(int N, const Dims& dims, const int32_t* __restrict__ idx, int64_t j,
                                           int64_t (&rows)[kMaxModes], int* status) {
    const int lane = threadIdx.x & 31;
    const int32_t my = lane < N ? idx[j * N + lane] : 0;
    const bool bad = lane < N && (my < 0 || (int64_t)my >= dims.d[lane]);
    if (__any_sync(0xffffffffu, bad)) {
        if (lane == 0 && status) atomicExch(status, 1);
        return false;
    }
#pragma unroll
    for (int k = 0; k < kMaxModes; k++) rows[k] = __shfl_sync(0xffffffffu, my, k);
    return true;
}

__device__ __forceinline__ double warp_sum_any(double v) { return warp_sum(v); }
__device__ __forceinline__ float warp_sum_any(float v) { return warp_sum(v); }

template <typename T>
__global__ void cp_model_kernel(int N, int R, Dims dims, int64_t J, const int32_t* __restrict__ idx,
                                PtrsT<const T> f, T* __restrict__ m, int* status) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = warp; j < J; j += nwarps) {
        int64_t rows[kMaxModes];
        if (!load_entry(N, dims, idx, j, rows, status)) {
            if (lane == 0) m[j] = T(0);
            continue;
        }
        T acc = 0;
        for (int c = lane; c < R; c += 32) {
            T p = 1;
#pragma unroll
            for (int k = 0; k < kMaxModes; k++)
                if (k < N) p *= f.p[k][rows[k] * R + c];
            acc += p;
        }
        acc = warp_sum_any(acc);
        if (lane == 0) m[j] = acc;
    }
}

template <typename T>
__global__ void cp_adjoint_kernel(int N, int R, Dims dims, int64_t J, const int32_t* __restrict__ idx,
                                  const T* __restrict__ gm, PtrsT<const T> f, PtrsT<T> g, int* status) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = warp; j < J; j += nwarps) {
        const T gj = gm[j];
        if (gj == T(0)) continue;  // uniform across the warp
        int64_t rows[kMaxModes];
        if (!load_entry(N, dims, idx, j, rows, status)) continue;
        for (int c = lane; c < R; c += 32) {
            T v[kMaxModes];
#pragma unroll
            for (int k = 0; k < kMaxModes; k++) v[k] = k < N ? f.p[k][rows[k] * R + c] : T(1);
#pragma unroll
            for (int n = 0; n < kMaxModes; n++) {
                if (n < N && g.p[n]) {
                    T p = gj;
#pragma unroll
                    for (int k = 0; k < kMaxModes; k++)
                        if (k < N && k != n) p *= v[k];
                    atomicAdd(&g.p[n][rows[n] * R + c], p);
                }
            }
        }
    }
}


template <typename T>
__global__ void gcp_sample_kernel(int N, Dims dims, int64_t nnz, const int32_t* __restrict__ nz_idx,
                                  const T* __restrict__ nz_vals, int64_t Jnz, int64_t Jz, uint64_t seed, uint64_t ctr,
                                  T wnz, T wz, int32_t* __restrict__ idx_out, T* __restrict__ x_out,
                                  T* __restrict__ w_out) {
    const int64_t J = Jnz + Jz;
    const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < J; j += (int64_t)gridDim.x * blockDim.x) {
        const uint4 r0 = philox4x32_10(make_uint4((unsigned)j, (unsigned)(j >> 32), (unsigned)ctr,
                                                  (unsigned)(ctr >> 32) ^ 0x9E3779B9u), key);
        if (j < Jnz) {
            // uniform nonzero: 64 random bits reduced modulo nnz (bias < nnz / 2^64)
            const uint64_t b = ((uint64_t)r0.x << 32) | r0.y;
            const int64_t e = (int64_t)(b % (uint64_t)nnz);
            for (int k = 0; k < N; k++) idx_out[j * N + k] = nz_idx[e * N + k];
            x_out[j] = nz_vals[e];
            w_out[j] = wnz;
        } else {
            // uniform coordinate, taken as a zero (a hit on a nonzero has
            // probability nnz / prod dims)
            const uint4 r1 = philox4x32_10(make_uint4((unsigned)j, (unsigned)(j >> 32), (unsigned)ctr,
                                                      (unsigned)(ctr >> 32) ^ 0x7F4A7C15u), key);
            const unsigned w8[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            for (int k = 0; k < N; k++) {
                const uint64_t b = ((uint64_t)w8[k] << 21) ^ (uint64_t)w8[(k + 4) & 7];
                idx_out[j * N + k] = (int32_t)(b % (uint64_t)dims.d[k]);
            }
            x_out[j] = T(0);
            w_out[j] = wz;
        }
    }
}

// Adam (Kingma and Ba; torch.optim.Adam's update without weight decay or
// amsgrad), per element in the parameter's own precision:
//   m = m + (1 - b1) (g - m);  v = b2 v + (1 - b2) g^2;
//   p = p - step_size m / (sqrt(v) / sqrt(1 - b2^t) + eps),  step_size = lr / (1 - b1^t)
// then p = max(p, lower) when projecting (a NaN stays NaN).  A null gradient
// counts as zero (the moments still decay and the parameter still moves).
struct AdamTensors {
    void* p[kMaxModes];
    const void* g[kMaxModes];
    void* m[kMaxModes];
    void* v[kMaxModes];
    int64_t n[kMaxModes];
};

template <typename T>
struct AdamCoef {
    T step_size, omb1, b2, omb2, bc2_sqrt, eps, lower;
    int project;
};

template <typename T>
__device__ __forceinline__ void adam_elem(T& p, T g, T& m, T& v, const AdamCoef<T>& c) {
    m = m + c.omb1 * (g - m);
    v = c.b2 * v + c.omb2 * (g * g);
    const T denom = sqrt(v) / c.bc2_sqrt + c.eps;
    p = p - c.step_size * (m / denom);
    if (c.project && p < c.lower) p = c.lower;
}

template <typename T, bool VEC>
__global__ void __launch_bounds__(256) adam_step_kernel(int count, AdamTensors ts, AdamCoef<T> c) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int t = 0; t < count; t++) {
        T* __restrict__ p = static_cast<T*>(ts.p[t]);
        const T* __restrict__ g = static_cast<const T*>(ts.g[t]);
        T* __restrict__ m = static_cast<T*>(ts.m[t]);
        T* __restrict__ v = static_cast<T*>(ts.v[t]);
        const int64_t n = ts.n[t];
        int64_t done = 0;
        if constexpr (VEC) {  // float4 body; every base is 16-byte aligned
            const int64_t nv = n >> 2;
            for (int64_t i = tid; i < nv; i += stride) {
                float4 P = reinterpret_cast<float4*>(p)[i];
                const float4 G = g ? reinterpret_cast<const float4*>(g)[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                float4 M = reinterpret_cast<float4*>(m)[i];
                float4 V = reinterpret_cast<float4*>(v)[i];
                adam_elem(P.x, G.x, M.x, V.x, c);
                adam_elem(P.y, G.y, M.y, V.y, c);
                adam_elem(P.z, G.z, M.z, V.z, c);
                adam_elem(P.w, G.w, M.w, V.w, c);
                reinterpret_cast<float4*>(p)[i] = P;
                reinterpret_cast<float4*>(m)[i] = M;
                reinterpret_cast<float4*>(v)[i] = V;
            }
            done = nv << 2;
        }
        for (int64_t i = done + tid; i < n; i += stride) {
            T P = p[i], M = m[i], V = v[i];
            adam_elem(P, g ? g[i] : T(0), M, V, c);
            p[i] = P;
            m[i] = M;
            v[i] = V;
        }
    }
}

static int grid_for(int64_t work, int per_block) {
    int64_t b = (work + per_block - 1) / per_block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace exafac

using namespace exafac;

#define GCP_DTYPE_ARG(dtype) \
    EXAFAC_ARG((dtype) == EXAFAC_DTYPE_F32 || (dtype) == EXAFAC_DTYPE_F64, "dtype must be EXAFAC_DTYPE_F32 or F64")

static int dims_arg(int N, const int64_t* dims, Dims* d) {
    EXAFAC_ARG(dims != nullptr, "null dims");
    for (int k = 0; k < kMaxModes; k++) d->d[k] = 0;
    for (int k = 0; k < N; k++) {
        EXAFAC_ARG(dims[k] >= 1 && dims[k] <= 0x7fffffffll, "mode sizes must be in [1, 2^31)");
        d->d[k] = dims[k];
    }
    return EXAFAC_OK;
}

extern "C" int exafac_cp_sampled_model(int32_t N, int32_t R, const int64_t* dims, int64_t J, const int32_t* idx,
                                       const void* const* factors, void* m_out, int32_t dtype, int32_t* status,
                                       void* stream) {
    EXAFAC_ARG(N >= 1 && N <= kMaxModes, "N must be in [1, 8]");
    EXAFAC_ARG(R >= 1, "R must be >= 1");
    EXAFAC_ARG(J >= 0, "J must be >= 0");
    GCP_DTYPE_ARG(dtype);
    Dims d;
    EXAFAC_TRY(dims_arg(N, dims, &d));
    if (J == 0) return EXAFAC_OK;
    EXAFAC_ARG(idx && factors && m_out, "null argument");
    for (int k = 0; k < N; k++) EXAFAC_ARG(factors[k] != nullptr, "null factor matrix");
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = grid_for(J, 8);
    if (dtype == EXAFAC_DTYPE_F32) {
        PtrsT<const float> f{};
        for (int k = 0; k < N; k++) f.p[k] = static_cast<const float*>(factors[k]);
        cp_model_kernel<float><<<grid, 256, 0, st>>>(N, R, d, J, idx, f, static_cast<float*>(m_out), status);
    } else {
        PtrsT<const double> f{};
        for (int k = 0; k < N; k++) f.p[k] = static_cast<const double*>(factors[k]);
        cp_model_kernel<double><<<grid, 256, 0, st>>>(N, R, d, J, idx, f, static_cast<double*>(m_out), status);
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

extern "C" int exafac_cp_sampled_adjoint(int32_t N, int32_t R, const int64_t* dims, int64_t J, const int32_t* idx,
                                         const void* grad_m, const void* const* factors, void* const* grads,
                                         int32_t dtype, int32_t* status, void* stream) {
    EXAFAC_ARG(N >= 1 && N <= kMaxModes, "N must be in [1, 8]");
    EXAFAC_ARG(R >= 1, "R must be >= 1");
    EXAFAC_ARG(J >= 0, "J must be >= 0");
    GCP_DTYPE_ARG(dtype);
    Dims d;
    EXAFAC_TRY(dims_arg(N, dims, &d));
    if (J == 0) return EXAFAC_OK;
    EXAFAC_ARG(idx && grad_m && factors && grads, "null argument");
    for (int k = 0; k < N; k++) EXAFAC_ARG(factors[k] != nullptr, "null factor matrix");
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = grid_for(J, 8);
    if (dtype == EXAFAC_DTYPE_F32) {
        PtrsT<const float> f{};
        PtrsT<float> g{};
        for (int k = 0; k < N; k++) {
            f.p[k] = static_cast<const float*>(factors[k]);
            g.p[k] = static_cast<float*>(grads[k]);
        }
        cp_adjoint_kernel<float><<<grid, 256, 0, st>>>(N, R, d, J, idx, static_cast<const float*>(grad_m), f, g,
                                                       status);
    } else {
        PtrsT<const double> f{};
        PtrsT<double> g{};
        for (int k = 0; k < N; k++) {
            f.p[k] = static_cast<const double*>(factors[k]);
            g.p[k] = static_cast<double*>(grads[k]);
        }
        cp_adjoint_kernel<double><<<grid, 256, 0, st>>>(N, R, d, J, idx, static_cast<const double*>(grad_m), f, g,
                                                        status);
    }
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

extern "C" int exafac_gcp_sample_entries(int32_t N, const int64_t* dims, int64_t nnz, const int32_t* nz_idx,
                                         const void* nz_vals, int64_t J_nz, int64_t J_z, uint64_t seed,
                                         uint64_t counter, int32_t* idx_out, void* x_out, void* w_out,
                                         int32_t dtype, void* stream) {
    EXAFAC_ARG(N >= 1 && N <= kMaxModes, "N must be in [1, 8]");
    EXAFAC_ARG(J_nz >= 0 && J_z >= 0, "sample counts must be >= 0");
    EXAFAC_ARG(J_nz == 0 || (nnz >= 1 && nz_idx && nz_vals), "nonzero samples need the nonzeros");
    GCP_DTYPE_ARG(dtype);
    Dims d;
    EXAFAC_TRY(dims_arg(N, dims, &d));
    if (J_nz + J_z == 0) return EXAFAC_OK;
    EXAFAC_ARG(idx_out && x_out && w_out, "null output");
    double total = 1.0;
    for (int k = 0; k < N; k++) total *= (double)dims[k];
    const double wnz = J_nz ? (double)nnz / (double)J_nz : 0.0;
    const double wz = J_z ? std::max(total - (double)nnz, 0.0) / (double)J_z : 0.0;
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = grid_for(J_nz + J_z, 256);
    if (dtype == EXAFAC_DTYPE_F32)
        gcp_sample_kernel<float><<<grid, 256, 0, st>>>(N, d, nnz, nz_idx, static_cast<const float*>(nz_vals), J_nz,
                                                       J_z, seed, counter, (float)wnz, (float)wz, idx_out,
                                                       static_cast<float*>(x_out), static_cast<float*>(w_out));
    else
        gcp_sample_kernel<double><<<grid, 256, 0, st>>>(N, d, nnz, nz_idx, static_cast<const double*>(nz_vals), J_nz,
                                                        J_z, seed, counter, wnz, wz, idx_out,
                                                        static_cast<double*>(x_out), static_cast<double*>(w_out));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

template <typename T>
static void launch_adam(int count, const AdamTensors& ts, int64_t total, double lr, double b1, double b2, double eps,
                        int64_t step, int project, double lower, bool vec, cudaStream_t st) {
    AdamCoef<T> c;
    c.step_size = (T)(lr / (1.0 - std::pow(b1, (double)step)));
    c.omb1 = (T)(1.0 - b1);
    c.b2 = (T)b2;
    c.omb2 = (T)(1.0 - b2);
    c.bc2_sqrt = (T)std::sqrt(1.0 - std::pow(b2, (double)step));
    c.eps = (T)eps;
    c.lower = (T)lower;
    c.project = project;
    const int grid = grid_for(vec ? (total + 3) / 4 : total, 256);
    if constexpr (std::is_same<T, float>::value) {
        if (vec) {
            adam_step_kernel<float, true><<<grid, 256, 0, st>>>(count, ts, c);
            return;
        }
    }
    adam_step_kernel<T, false><<<grid, 256, 0, st>>>(count, ts, c);
}

extern "C" int exafac_adam_step(int32_t count, void* const* params, const void* const* grads, void* const* exp_avg,
                                void* const* exp_avg_sq, const int64_t* numel, int32_t dtype, double lr,
                                double beta1, double beta2, double eps, int64_t step, int32_t project, double lower,
                                void* stream) {
    EXAFAC_ARG(count >= 0 && count <= kMaxModes, "count must be in [0, 8]");
    GCP_DTYPE_ARG(dtype);
    EXAFAC_ARG(step >= 1, "step must be >= 1 (the step count after this update)");
    EXAFAC_ARG(beta1 >= 0.0 && beta1 < 1.0 && beta2 >= 0.0 && beta2 < 1.0, "betas must be in [0, 1)");
    EXAFAC_ARG(eps >= 0.0 && lr >= 0.0, "lr and eps must be >= 0");
    if (count == 0) return EXAFAC_OK;
    EXAFAC_ARG(params && exp_avg && exp_avg_sq && numel, "null argument");
    AdamTensors ts{};
    int64_t total = 0;
    bool vec = dtype == EXAFAC_DTYPE_F32;
    for (int t = 0; t < count; t++) {
        EXAFAC_ARG(numel[t] >= 0, "element counts must be >= 0");
        EXAFAC_ARG(numel[t] == 0 || (params[t] && exp_avg[t] && exp_avg_sq[t]), "null parameter or moment");
        ts.p[t] = params[t];
        ts.g[t] = grads ? grads[t] : nullptr;
        ts.m[t] = exp_avg[t];
        ts.v[t] = exp_avg_sq[t];
        ts.n[t] = numel[t];
        total = std::max<int64_t>(total, numel[t]);
        const uintptr_t a = (uintptr_t)ts.p[t] | (uintptr_t)ts.g[t] | (uintptr_t)ts.m[t] | (uintptr_t)ts.v[t];
        if (a & 15u) vec = false;
    }
    if (total == 0) return EXAFAC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == EXAFAC_DTYPE_F32)
        launch_adam<float>(count, ts, total, lr, beta1, beta2, eps, step, project, lower, vec, st);
    else
        launch_adam<double>(count, ts, total, lr, beta1, beta2, eps, step, project, lower, false, st);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

