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
//
// The adjoint accumulates with atomic adds, so its last bits depend on the
// order in which entries that share a row arrive.
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
