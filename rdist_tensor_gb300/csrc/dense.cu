// Small dense FP64 R x R algebra: symmetric eigendecomposition (parallel
// cyclic Jacobi, one CTA per matrix) and the symmetric pseudo-inverse built
// on it.  Replaces LAPACKE_dsyev + compute_pinv_square (common.h:405-443,
// sts_cp.hpp:110-176) of the reference.
#include "dense.cuh"

namespace exafac {

// Round-robin ("circle") pairing of Re = even(R) indices: in round t, pair 0
// is (0, 1 + t mod m) and pair i >= 1 is (1 + (t+i) mod m, 1 + (t-i) mod m),
// m = Re - 1.  Every unordered pair meets once per sweep of Re - 1 rounds.
__device__ __forceinline__ void rr_pair(int t, int i, int m, int& p, int& q) {
    if (i == 0) {
        p = 0;
        q = 1 + (t % m);
    } else {
        p = 1 + ((t + i) % m);
        q = 1 + ((t - i + m * 4) % m);
    }
    if (p > q) {
        int x = p;
        p = q;
        q = x;
    }
}

// Jacobi on the symmetric matrix whose upper triangle is A (row-major R x R).
// Shared: a[Re*Re] (the working matrix), rot[Re/2] cosines and sines.
// vt (global, Re*Re) holds V^T: vt[i*Re + r] = component r of eigenvector i.
__device__ void jacobi_block(int R, const double* __restrict__ A, double* a, double* vt, double* rc, double* rs,
                             int* flag) {
    const int Re = R + (R & 1);
    const int m = Re - 1;
    const int npairs = Re / 2;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < Re * Re; e += nt) {
        int i = e / Re, j = e % Re;
        double v = 0.0;
        if (i < R && j < R) v = (i <= j) ? A[i * R + j] : A[j * R + i];
        a[e] = v;
        vt[e] = (i == j && i < R) ? 1.0 : 0.0;
    }
    __syncthreads();
    if (R == 1) return;
    for (int sweep = 0; sweep < 60; sweep++) {
        if (tid == 0) *flag = 0;
        __syncthreads();
        for (int t = 0; t < m; t++) {
            // Rotation angles (Golub & Van Loan, sym.schur2).
            for (int i = tid; i < npairs; i += nt) {
                int p, q;
                rr_pair(t, i, m, p, q);
                double c = 1.0, s = 0.0;
                if (q < R) {
                    double apq = a[p * Re + q];
                    double app = a[p * Re + p], aqq = a[q * Re + q];
                    if (apq != 0.0 && fabs(apq) > 1e-18 * sqrt(fabs(app * aqq))) {
                        double tau = (aqq - app) / (2.0 * apq);
                        double tt;
                        if (fabs(tau) > 1e150) {
                            tt = 0.5 / tau;
                        } else {
                            tt = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        }
                        c = 1.0 / sqrt(1.0 + tt * tt);
                        s = tt * c;
                        *flag = 1;
                    }
                }
                rc[i] = c;
                rs[i] = s;
            }
            __syncthreads();
            // B = J^T A: rows p, q.
            for (int e = tid; e < npairs * Re; e += nt) {
                int i = e / Re, col = e % Re;
                double s = rs[i];
                if (s == 0.0) continue;
                double c = rc[i];
                int p, q;
                rr_pair(t, i, m, p, q);
                double ap = a[p * Re + col], aq = a[q * Re + col];
                a[p * Re + col] = c * ap - s * aq;
                a[q * Re + col] = s * ap + c * aq;
            }
            __syncthreads();
            // A' = B J and V' = V J: columns p, q.
            for (int e = tid; e < npairs * Re; e += nt) {
                int i = e / Re, row = e % Re;
                double s = rs[i];
                if (s == 0.0) continue;
                double c = rc[i];
                int p, q;
                rr_pair(t, i, m, p, q);
                double bp = a[row * Re + p], bq = a[row * Re + q];
                a[row * Re + p] = c * bp - s * bq;
                a[row * Re + q] = s * bp + c * bq;
                double vp = vt[p * Re + row], vq = vt[q * Re + row];
                vt[p * Re + row] = c * vp - s * vq;
                vt[q * Re + row] = s * vp + c * vq;
            }
            __syncthreads();
        }
        if (*flag == 0) break;
        __syncthreads();
    }
}

// Ascending order of the diagonal: rank[i] = #{j : d_j < d_i or (d_j == d_i and j < i)}.
__device__ void ascending_ranks(int R, const double* a, int Re, int* rank) {
    for (int i = threadIdx.x; i < R; i += blockDim.x) {
        double di = a[i * Re + i];
        int r = 0;
        for (int j = 0; j < R; j++) {
            double dj = a[j * Re + j];
            r += (dj < di) || (dj == di && j < i);
        }
        rank[i] = r;
    }
}

// One CTA per matrix.  Outputs (any may be null):
//   V[u*R + v]    eigenvector v (ascending eigenvalues), lam[v]
//   pinv          sum over lam_v > tol of v v^T / lam_v  (full symmetric)
__global__ void syev_kernel(int R, const double* __restrict__ A, int64_t a_stride, double* V, double* lam,
                            int64_t v_stride, double* pinv, double tol, double* vt_scratch) {
    extern __shared__ double smem[];
    const int Re = R + (R & 1);
    double* a = smem;
    double* rc = a + Re * Re;
    double* rs = rc + Re / 2 + 1;
    int* rank = reinterpret_cast<int*>(rs + Re / 2 + 1);
    int* order = rank + Re;
    int* flag = order + Re;
    const int b = blockIdx.x;
    double* vt = vt_scratch + (int64_t)b * Re * Re;
    jacobi_block(R, A + b * a_stride, a, vt, rc, rs, flag);
    __syncthreads();
    ascending_ranks(R, a, Re, rank);
    __syncthreads();
    for (int i = threadIdx.x; i < R; i += blockDim.x) order[rank[i]] = i;
    __syncthreads();
    if (V) {
        for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
            int i = e / R, u = e % R;  // eigenvector i (original slot), component u
            V[b * v_stride + u * R + rank[i]] = vt[i * Re + u];
        }
    }
    if (lam) {
        for (int i = threadIdx.x; i < R; i += blockDim.x) lam[b * R + rank[i]] = a[i * Re + i];
    }
    if (pinv) {
        // Sum over eigen-pairs in ascending eigenvalue order, as
        // (V L^-1/2)(V L^-1/2)^T accumulates in the reference's dsyrk.
        for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
            int r1 = e / R, r2 = e % R;
            double acc = 0.0;
            for (int k = 0; k < R; k++) {
                int i = order[k];
                double l = a[i * Re + i];
                if (l > tol) {
                    double s = 1.0 / sqrt(l);
                    acc += (vt[i * Re + r1] * s) * (vt[i * Re + r2] * s);
                }
            }
            pinv[b * (int64_t)R * R + e] = acc;
        }
    }
}

size_t syev_smem_bytes(int R) {
    int Re = R + (R & 1);
    return sizeof(double) * ((size_t)Re * Re + Re + 2) + sizeof(int) * (2 * Re + 1) + 16;
}

size_t syev_scratch_doubles(int R, int batch) {
    int Re = R + (R & 1);
    return (size_t)batch * Re * Re;
}

int launch_syev(int R, const double* A, int64_t a_stride, int batch, double* V, double* lam, int64_t v_stride,
                double* pinv, double tol, double* vt_scratch, cudaStream_t stream) {
    size_t smem = syev_smem_bytes(R);
    if (smem > 48 * 1024) {
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(syev_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    int threads = R <= 32 ? 256 : 512;
    syev_kernel<<<batch, threads, smem, stream>>>(R, A, a_stride, V, lam, v_stride, pinv, tol, vt_scratch); count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

}  // namespace exafac

using namespace exafac;

extern "C" size_t exafac_dense_workspace_bytes(int32_t R) {
    if (R < 1 || R > kMaxRank) return 0;
    return sizeof(double) * syev_scratch_doubles(R, 1);
}

extern "C" int exafac_syev(int32_t R, const double* A, double* V, double* lam, void* workspace, size_t workspace_bytes,
                           void* stream) {
    EXAFAC_ARG(R >= 1 && R <= kMaxRank, "exafac_syev: R out of range");
    EXAFAC_ARG(A && V && lam && workspace, "exafac_syev: null pointer");
    EXAFAC_ARG(workspace_bytes >= exafac_dense_workspace_bytes(R), "exafac_syev: workspace too small");
    return launch_syev(R, A, 0, 1, V, lam, 0, nullptr, 0.0, (double*)workspace, (cudaStream_t)stream);
}

extern "C" int exafac_pinv_square(int32_t R, const double* A, double* out, double tol, void* workspace,
                                  size_t workspace_bytes, void* stream) {
    EXAFAC_ARG(R >= 1 && R <= kMaxRank, "exafac_pinv_square: R out of range");
    EXAFAC_ARG(A && out && workspace, "exafac_pinv_square: null pointer");
    EXAFAC_ARG(workspace_bytes >= exafac_dense_workspace_bytes(R), "exafac_pinv_square: workspace too small");
    return launch_syev(R, A, 0, 1, nullptr, nullptr, 0, out, tol, (double*)workspace, (cudaStream_t)stream);
}
