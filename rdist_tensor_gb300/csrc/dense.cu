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
                    // Rotate unless a_pq is negligible relative to the
                    // diagonal (Demmel-Veselic criterion, tol = R * eps).
                    if (apq != 0.0 && fabs(apq) > (double)R * 2.220446049250313e-16 * sqrt(fabs(app * aqq))) {
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

// Ascending order of the diagonal: rank[i] = #{j : d_j before d_i}, with
// "before" a strict total order (value, then index; NaNs after every number),
// so the ranks are a permutation of 0..R-1 whatever the values: the order[]
// built from them has no unwritten slot even when a NaN reached the matrix.
__device__ __forceinline__ bool diag_before(double dj, int j, double di, int i) {
    const bool nj = isnan(dj), ni = isnan(di);
    if (nj || ni) return nj == ni ? j < i : ni;
    return dj < di || (dj == di && j < i);
}
__device__ void ascending_ranks(int R, const double* a, int Re, int* rank) {
    for (int i = threadIdx.x; i < R; i += blockDim.x) {
        const double di = a[i * Re + i];
        int r = 0;
        for (int j = 0; j < R; j++) r += diag_before(a[j * Re + j], j, di, i);
        rank[i] = r;
    }
}

// Eigendecomposition / pseudo-inverse of one matrix by the calling CTA.
// Outputs (any may be null):
//   V[u*R + v]    eigenvector v (ascending eigenvalues), lam[v]
//   pinv          sum over lam_v > tol of v v^T / lam_v  (full symmetric)
__device__ void syev_block(int R, const double* __restrict__ A, double* V, double* lam, double* pinv, double tol,
                           double* vt, double* smem) {
    const int Re = R + (R & 1);
    double* a = smem;
    double* rc = a + Re * Re;
    double* rs = rc + Re / 2 + 1;
    int* rank = reinterpret_cast<int*>(rs + Re / 2 + 1);
    int* order = rank + Re;
    int* flag = order + Re;
    const int b = 0;
    const int64_t v_stride = 0;
    jacobi_block(R, A, a, vt, rc, rs, flag);
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

// One CTA per matrix (matrix b at A + b * a_stride).
__global__ void syev_kernel(int R, const double* __restrict__ A, int64_t a_stride, double* V, double* lam,
                            int64_t v_stride, double* pinv, double tol, double* vt_scratch) {
    extern __shared__ double smem[];
    const int Re = R + (R & 1);
    const int b = blockIdx.x;
    syev_block(R, A + b * a_stride, V ? V + b * v_stride : nullptr, lam ? lam + (int64_t)b * R : nullptr,
               pinv ? pinv + (int64_t)b * R * R : nullptr, tol, vt_scratch + (int64_t)b * Re * Re, smem);
}

// Symmetric pseudo-inverse, fast path: Cholesky A = L L^T, L^{-1} by
// substitution, A^{-1} = L^{-T} L^{-1}.  A^{-1} equals the thresholded
// pseudo-inverse when every eigenvalue exceeds tol; the path is taken only
// when lambda_min >= 1 / ||A^{-1}||_F > 10 tol (a guaranteed lower bound,
// with margin for rounding).  Otherwise — not positive definite, or possibly
// an eigenvalue near or below tol — the same CTA computes the Jacobi
// pseudo-inverse (compute_pinv_square semantics).
// One Newton step on an (pseudo-)inverse X of A: X <- 2X - X A X, in FP64.
// A pseudo-inverse is a fixed point of the step.  smem: 3 R^2 doubles.
__device__ void newton_refine(int R, const double* __restrict__ A, double* __restrict__ out, double* smem) {
    double* X = smem;
    double* As = smem + R * R;
    double* T = smem + 2 * R * R;
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        X[e] = out[e];
        int i = e / R, j = e % R;
        As[e] = (i <= j) ? A[i * R + j] : A[j * R + i];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {  // T = A X
        int i = e / R, j = e % R;
        double acc = 0.0;
        for (int k = 0; k < R; k++) acc = fma(As[i * R + k], X[k * R + j], acc);
        T[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {  // out = 2X - X T
        int i = e / R, j = e % R;
        double acc = 0.0;
        for (int k = 0; k < R; k++) acc = fma(X[i * R + k], T[k * R + j], acc);
        out[e] = 2.0 * X[e] - acc;
    }
    __syncthreads();
}

__global__ void spd_pinv_kernel(int R, const double* __restrict__ A, double* __restrict__ out, double tol,
                                double* vt_scratch, int refine, int fast) {
    extern __shared__ double smem[];
    __shared__ int fail;
    __shared__ double fro;
    __shared__ double fro_w[32];  // per-warp parts, summed in warp order (no atomics: the result repeats)
    double* L = smem;
    double* Li = smem + R * R;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (!fast) {  // the Cholesky buffers do not fit in shared memory
        syev_block(R, A, nullptr, nullptr, out, tol, vt_scratch, smem);
        return;
    }
    for (int e = tid; e < R * R; e += nt) {
        int i = e / R, j = e % R;
        L[e] = (i <= j) ? A[i * R + j] : A[j * R + i];
        Li[e] = 0.0;
    }
    if (tid == 0) {
        fail = 0;
        fro = 0.0;
    }
    __syncthreads();
    for (int k = 0; k < R; k++) {
        if (tid == 0) {
            double d = L[k * R + k];
            if (!(d > 0.0) || !isfinite(d)) fail = 1;
            else L[k * R + k] = sqrt(d);
        }
        __syncthreads();
        if (fail) break;
        const double lkk = L[k * R + k];
        for (int i = k + 1 + tid; i < R; i += nt) L[i * R + k] /= lkk;
        __syncthreads();
        const int m = R - k - 1;
        for (int e = tid; e < m * m; e += nt) {
            int i = k + 1 + e / m, j = k + 1 + e % m;
            if (j <= i) L[i * R + j] -= L[i * R + k] * L[j * R + k];
        }
        __syncthreads();
    }
    if (!fail) {
        for (int c = tid; c < R; c += nt) {
            for (int i = c; i < R; i++) {
                double s = (i == c) ? 1.0 : 0.0;
                for (int t = c; t < i; t++) s -= L[i * R + t] * Li[t * R + c];
                Li[i * R + c] = s / L[i * R + i];
            }
        }
        __syncthreads();
        double part = 0.0;
        for (int e = tid; e < R * R; e += nt) {
            int a = e / R, b = e % R;
            int k0 = a > b ? a : b;
            double acc = 0.0;
            for (int k = k0; k < R; k++) acc = fma(Li[k * R + a], Li[k * R + b], acc);
            out[e] = acc;
            part += acc * acc;
        }
        part = warp_sum(part);
        if ((tid & 31) == 0) fro_w[tid >> 5] = part;
        __syncthreads();
        if (tid == 0) {
            double f = 0.0;
            for (int q = 0; q < (nt + 31) / 32; q++) f += fro_w[q];
            fro = f;
        }
        __syncthreads();
        const double bound = 1.0 / sqrt(fro);
        if (isfinite(fro) && bound > 10.0 * tol) {
            if (refine) newton_refine(R, A, out, smem);
            return;
        }
        __syncthreads();
    }
    syev_block(R, A, nullptr, nullptr, out, tol, vt_scratch, smem);
    if (refine) newton_refine(R, A, out, smem);
}

// R <= 32: the symmetric sweep operator (Gauss-Jordan with diagonal pivots,
// stable without pivoting on a positive-definite matrix) with the upper
// triangle held in registers, kSmallPinvEpt elements per thread.  Sweeping
// every pivot leaves -A^{-1}.  A non-positive pivot means A is not positive
// definite.  The same acceptance test as the Cholesky path (lambda_min >=
// 1/||A^{-1}||_F > 10 tol) guards the result; otherwise the CTA computes the
// Jacobi pseudo-inverse.
//
// Per pivot, warp 0 forms 1/pivot and the scaled pivot row once (one FP64
// division per pivot, not one per thread: GB300 retires about two FP64
// operations per clock per SM), then every element takes one FMA.
//
// refine == 2 tries pinv_sweep_f32 first (below).  The refinement (refine
// == 1) is the Newton step written as
// X + X (I - A X): the residual I - A X is formed in FP64 (A staged in shared
// memory) and the small correction X (I - A X) in FP32 from FP32 copies of X
// and the residual, which keeps the FP64 pipe to a single R^3 product.
constexpr int kSmallPinvThreads = 128;
constexpr int kSmallPinvMaxR = 32;
constexpr int kSmallPinvEpt = (kSmallPinvMaxR * (kSmallPinvMaxR + 1) / 2 + kSmallPinvThreads - 1) / kSmallPinvThreads;

// The same sweep in FP32 (mode 2: the leverage-score pseudo-inverse of the
// mixed forms, whose scores are formed in FP32 anyway), run by warp 0 with
// the whole matrix in registers.  Lane j holds column j; the rows rotate
// through the registers so that the pivot row is always slot 0 (before pivot
// k, slot s holds row (k + s) mod 32), which keeps every register index
// static in a rolled pivot loop.  The swept matrix stays symmetric, so the
// pivot column's entry for row (k + s) is lane (k + s)'s row-k value, one
// shuffle each; no barrier per pivot.  Rows and lanes >= R hold zeros and
// stay zero.  Accepted when every pivot is positive and the FP32 error bound
// R ||A^{-1}||_F 2^-24 (A has a unit diagonal here, so R bounds ||A||) stays
// below 2^-10; otherwise the caller falls back to the FP64 sweep.  A
// dependent FP64 operation costs ~64 cycles on GB300 against ~4 for FP32, and
// this inverse sits on the step's critical path.  Returns the block-uniform
// accept flag; on acceptance out holds the inverse.
__device__ bool pinv_sweep_f32(int R, const double* __restrict__ A, double* __restrict__ out) {
    // Loads, conversions and stores run as rolled loops over the whole block:
    // a single warp's straight-line code is fetched once and pays the
    // instruction-fetch latency per line.
    __shared__ float Af[32][33];
    __shared__ int accepted;
    const int tid = threadIdx.x;
    for (int e = tid; e < 32 * 32; e += blockDim.x) {
        const int i = e >> 5, c = e & 31;
        Af[i][c] = (i < R && c < R) ? narrow_f64(A[i * R + c]) : 0.0f;
    }
    __syncthreads();
    if (tid < 32) {
        const int j = tid;
        const unsigned full = 0xffffffffu;
        float col[32];
#pragma unroll
        for (int s = 0; s < 32; s++) col[s] = Af[s][j];
        bool ok = true;
#pragma unroll 1
        for (int k = 0; k < R; k++) {
            const float akj = col[0];                     // A[k][j]
            const float piv = __shfl_sync(full, akj, k);  // A[k][k], the same in every lane
            if (!(piv > 0.0f) || !isfinite(piv)) {
                ok = false;
                break;
            }
            const float p = 1.0f / piv;
            const float akjp = akj * p;
            float nxt[32];
#pragma unroll
            for (int s = 1; s < 32; s++) {
                const float aik = __shfl_sync(full, akj, (k + s) & 31);  // A[k + s][k]
                nxt[s - 1] = (j == k) ? aik * p : fmaf(-aik, akjp, col[s]);
            }
            nxt[31] = (j == k) ? -p : akjp;  // row k moves to the last slot
#pragma unroll
            for (int s = 0; s < 32; s++) col[s] = nxt[s];
        }
        float fro = 0.0f;
#pragma unroll
        for (int s = 0; s < 32; s++) fro = fmaf(col[s], col[s], fro);
        fro = warp_sum(fro);
        ok = ok && isfinite(fro) && (float)R * sqrtf(fro) <= 0x1.0p14f;  // R ||X||_F 2^-24 <= 2^-10
        __syncwarp();
#pragma unroll
        for (int s = 0; s < 32; s++) Af[(R + s) & 31][j] = -col[s];  // after R pivots slot s holds row (R + s) mod 32
        if (j == 0) accepted = ok;
    }
    __syncthreads();
    if (!accepted) return false;
    for (int e = tid; e < R * R; e += blockDim.x) out[e] = widen_f32(Af[e / R][e % R]);
    return true;
}

__device__ void pinv_small_block(int R, const double* __restrict__ A, double* __restrict__ out, double tol,
                                 double* vt_scratch, int refine) {
    extern __shared__ double smem[];  // Jacobi fallback; in the accepted path A, X and E staged for refinement
    __shared__ double rowbuf[2][kSmallPinvMaxR];  // pivot row k (unscaled), ping-pong
    __shared__ double rp[kSmallPinvMaxR];         // pivot row k times 1/pivot
    __shared__ double pinv_k;                     // 1/pivot
    __shared__ int bad;
    __shared__ double Xs[kSmallPinvMaxR][kSmallPinvMaxR + 1];
    __shared__ double fro;
    __shared__ double fro_w[kSmallPinvThreads / 32];  // per-warp parts, summed in warp order
    if (refine == 2 && pinv_sweep_f32(R, A, out)) return;
    const int tid = threadIdx.x;
    const int P = R * (R + 1) / 2;
    int ii[kSmallPinvEpt], jj[kSmallPinvEpt];
    double a[kSmallPinvEpt];
#pragma unroll
    for (int m = 0; m < kSmallPinvEpt; m++) {
        const int e = tid + kSmallPinvThreads * m;
        int i = 0, base = 0;
        while (i < R - 1 && e >= base + (R - i)) {
            base += R - i;
            i++;
        }
        ii[m] = (e < P) ? i : -1;
        jj[m] = (e < P) ? i + (e - base) : -1;
        a[m] = (e < P) ? A[i * R + jj[m]] : 0.0;
    }
    if (tid < R) rowbuf[0][tid] = A[tid];
    if (tid == 0) {
        fro = 0.0;
        bad = 0;
    }
    __syncthreads();
    bool ok = true;
    for (int k = 0; k < R; k++) {
        const double* r = rowbuf[k & 1];
        double* nr = rowbuf[(k + 1) & 1];
        if (tid < 32) {
            const double piv = r[k];
            if (!(piv > 0.0) || !isfinite(piv)) {
                if (tid == 0) bad = 1;
            } else {
                const double p = 1.0 / piv;
                if (tid < R) rp[tid] = r[tid] * p;
                if (tid == 0) pinv_k = p;
            }
        }
        __syncthreads();
        if (bad) {  // uniform
            ok = false;
            break;
        }
        const double p = pinv_k;
#pragma unroll
        for (int m = 0; m < kSmallPinvEpt; m++) {
            const int i = ii[m], j = jj[m];
            if (i < 0) continue;
            double v;
            if (i != k && j != k) v = fma(-rp[i], r[j], a[m]);
            else if (i == k && j == k) v = -p;
            else v = rp[i == k ? j : i];
            a[m] = v;
            if (i == k + 1) nr[j] = v;
            else if (j == k + 1) nr[i] = v;
        }
        __syncthreads();
    }
    if (ok) {
        double part = 0.0;
#pragma unroll
        for (int m = 0; m < kSmallPinvEpt; m++) {
            if (ii[m] < 0) continue;
            const double x = -a[m];
            a[m] = x;
            part += (ii[m] == jj[m] ? 1.0 : 2.0) * x * x;
            Xs[ii[m]][jj[m]] = x;
            Xs[jj[m]][ii[m]] = x;
        }
        part = warp_sum(part);
        if ((tid & 31) == 0) fro_w[tid >> 5] = part;
        __syncthreads();
        if (tid == 0) {
            double f = 0.0;
            for (int q = 0; q < kSmallPinvThreads / 32; q++) f += fro_w[q];
            fro = f;
        }
        __syncthreads();
        ok = isfinite(fro) && 1.0 / sqrt(fro) > 10.0 * tol;
    }
    if (ok) {
        if (refine != 1) {
            for (int e = tid; e < R * R; e += kSmallPinvThreads) out[e] = Xs[e / R][e % R];
            return;
        }
        double* As = smem;                                        // R x R
        float* Xf = reinterpret_cast<float*>(smem + R * R);       // R x (R + 1)
        float* Ef = Xf + R * (R + 1);                             // R x (R + 1)
        for (int e = tid; e < R * R; e += kSmallPinvThreads) {
            const int i = e / R, j = e % R;
            As[e] = A[(i <= j) ? i * R + j : j * R + i];
            Xf[i * (R + 1) + j] = narrow_f64(Xs[i][j]);
        }
        __syncthreads();
        for (int e = tid; e < R * R; e += kSmallPinvThreads) {  // E = I - A X
            const int i = e / R, j = e % R;
            double acc = (i == j) ? 1.0 : 0.0;
            for (int t = 0; t < R; t++) acc = fma(-As[i * R + t], Xs[t][j], acc);
            Ef[i * (R + 1) + j] = narrow_f64(acc);
        }
        __syncthreads();
        for (int e = tid; e < R * R; e += kSmallPinvThreads) {  // out = X + X E
            const int i = e / R, j = e % R;
            float c = 0.0f;
            for (int t = 0; t < R; t++) c = fmaf(Xf[i * (R + 1) + t], Ef[t * (R + 1) + j], c);
            out[e] = Xs[i][j] + widen_f32(c);
        }
        return;
    }
    __syncthreads();
    syev_block(R, A, nullptr, nullptr, out, tol, vt_scratch, smem);
    if (refine == 1) newton_refine(R, A, out, smem);
}

__global__ void __launch_bounds__(kSmallPinvThreads)
    spd_pinv_small_kernel(int R, const double* __restrict__ A, double* __restrict__ out, double tol,
                          double* vt_scratch, int refine) {
    pinv_small_block(R, A, out, tol, vt_scratch, refine);
}

// The mixed forms' normalisation head in one block: column norms sigma_c =
// sqrt(G_cc) of the factor Gram (DistMat1D::renormalize_columns,
// distmat.hpp:85-138), the normalised Gram ngram = G_ab / (sigma_a sigma_b)
// (as products with 1 / sigma: the leverage inverse is an FP32 quantity),
// the degenerate flag, then the leverage pseudo-inverse of ngram (FP32 sweep
// first).
__global__ void __launch_bounds__(kSmallPinvThreads)
    sigma_pinv_kernel(int R, const double* __restrict__ ugram, double* __restrict__ sigma,
                      double* __restrict__ ngram, int* __restrict__ degenerate, double* __restrict__ out, double tol,
                      double* vt_scratch) {
    __shared__ double rinv[kSmallPinvMaxR];
    __shared__ int deg;
    pdl_wait();
    pdl_trigger();
    if (threadIdx.x == 0) deg = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < R; c += blockDim.x) {
        const double v = sqrt(ugram[c * R + c]);
        sigma[c] = v;
        rinv[c] = 1.0 / v;
        if (!(v > 0.0)) deg = 1;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) ngram[e] = ugram[e] * rinv[e / R] * rinv[e % R];
    if (threadIdx.x == 0) *degenerate = deg;
    __syncthreads();  // the block's writes of ngram are visible to it
    pinv_small_block(R, ngram, out, tol, vt_scratch, 2);
}

// Larger ranks (R > 92, where three full R x R matrices pass the shared
// memory cap): the same Cholesky inverse with L and L^{-1} held as packed
// lower triangles ((i, j), j <= i, at i (i + 1) / 2 + j; two times 66 KB at
// R = 128), the same acceptance test and Jacobi fallback; the Newton step,
// when asked for, runs in global scratch (2 R^2 doubles of vt_scratch: the
// sessions' scratch holds (N + 1) R^2).
__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// Sums with four independent FP64 accumulators (a dependent FP64 operation
// takes ~64 cycles on GB300, so one chain of R FMAs is latency-bound).
// sub_dot: s0 - sum_{t in [t0, t1)} L(i, t) Li(t, c); gram_dot: sum_{k in
// [k0, R)} Li(k, a) Li(k, b); both over packed lower triangles.
__device__ __forceinline__ double sub_dot(const double* L, const double* Li, int i, int c, int t0, int t1,
                                          double s0) {
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int t = t0;
    for (; t + 3 < t1; t += 4) {
        s0 -= L[tri(i, t)] * Li[tri(t, c)];
        s1 -= L[tri(i, t + 1)] * Li[tri(t + 1, c)];
        s2 -= L[tri(i, t + 2)] * Li[tri(t + 2, c)];
        s3 -= L[tri(i, t + 3)] * Li[tri(t + 3, c)];
    }
    for (; t < t1; t++) s0 -= L[tri(i, t)] * Li[tri(t, c)];
    return (s0 + s1) + (s2 + s3);
}
__device__ __forceinline__ double gram_dot(const double* Li, int a, int b, int k0, int R) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int k = k0;
    for (; k + 3 < R; k += 4) {
        s0 = fma(Li[tri(k, a)], Li[tri(k, b)], s0);
        s1 = fma(Li[tri(k + 1, a)], Li[tri(k + 1, b)], s1);
        s2 = fma(Li[tri(k + 2, a)], Li[tri(k + 2, b)], s2);
        s3 = fma(Li[tri(k + 3, a)], Li[tri(k + 3, b)], s3);
    }
    for (; k < R; k++) s0 = fma(Li[tri(k, a)], Li[tri(k, b)], s0);
    return (s0 + s1) + (s2 + s3);
}

__device__ void newton_refine_global(int R, const double* __restrict__ A, double* __restrict__ out,
                                     double* __restrict__ scratch) {
    double* X = scratch;
    double* T = scratch + (size_t)R * R;
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) X[e] = out[e];
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {  // T = A X
        const int i = e / R, j = e % R;
        double acc = 0.0;
        for (int k = 0; k < R; k++) acc = fma(i <= k ? A[i * R + k] : A[k * R + i], X[k * R + j], acc);
        T[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {  // out = 2X - X T
        const int i = e / R, j = e % R;
        double acc = 0.0;
        for (int k = 0; k < R; k++) acc = fma(X[i * R + k], T[k * R + j], acc);
        out[e] = 2.0 * X[e] - acc;
    }
    __syncthreads();
}

__global__ void spd_pinv_packed_kernel(int R, const double* __restrict__ A, double* __restrict__ out, double tol,
                                       double* vt_scratch, int refine) {
    extern __shared__ double smem[];
    __shared__ int fail;
    __shared__ double fro_w[32];  // per-warp parts, summed in warp order
    const int P = R * (R + 1) / 2;
    double* L = smem;
    double* Li = smem + P;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < R; i += nt)
        for (int j = 0; j <= i; j++) {
            L[tri(i, j)] = A[j * R + i];  // upper triangle of A
            Li[tri(i, j)] = 0.0;
        }
    if (tid == 0) fail = 0;
    __syncthreads();
    for (int k = 0; k < R; k++) {
        if (tid == 0) {
            const double d = L[tri(k, k)];
            if (!(d > 0.0) || !isfinite(d)) fail = 1;
            else L[tri(k, k)] = sqrt(d);
        }
        __syncthreads();
        if (fail) break;
        const double lkk = L[tri(k, k)];
        for (int i = k + 1 + tid; i < R; i += nt) L[tri(i, k)] /= lkk;
        __syncthreads();
        {  // the trailing lower triangle: a warp per row, its lanes along the row
            const int wid = tid >> 5, lane = tid & 31, nw = nt >> 5;
            for (int i = k + 1 + wid; i < R; i += nw) {
                const double lik = L[tri(i, k)];
                double* row = L + tri(i, 0);
                for (int j = k + 1 + lane; j <= i; j += 32) row[j] -= lik * L[tri(j, k)];
            }
        }
        __syncthreads();
    }
    if (!fail) {
        for (int c = tid; c < R; c += nt) {
            for (int i = c; i < R; i++) {
                const double sacc = sub_dot(L, Li, i, c, c, i, (i == c) ? 1.0 : 0.0);
                Li[tri(i, c)] = sacc / L[tri(i, i)];
            }
        }
        __syncthreads();
        double part = 0.0;
        for (int e = tid; e < R * R; e += nt) {  // (a, b), a <= b, computed once and mirrored
            const int a = e / R, b = e % R;
            if (a > b) continue;
            const double acc = gram_dot(Li, a, b, b, R);
            out[a * R + b] = acc;
            out[b * R + a] = acc;
            part += (a == b ? 1.0 : 2.0) * (acc * acc);
        }
        part = warp_sum(part);
        if ((tid & 31) == 0) fro_w[tid >> 5] = part;
        __syncthreads();
        double fro = 0.0;
        for (int q = 0; q < (nt + 31) / 32; q++) fro += fro_w[q];
        const double bound = 1.0 / sqrt(fro);
        if (isfinite(fro) && bound > 10.0 * tol) {  // the same in every thread
            if (refine) newton_refine_global(R, A, out, vt_scratch);
            return;
        }
        __syncthreads();
    }
    syev_block(R, A, nullptr, nullptr, out, tol, vt_scratch, smem);
    if (refine) newton_refine_global(R, A, out, vt_scratch);
}

// The Newton step X <- X + X (I - A X) (= 2X - X A X, the fixed point a
// pseudo-inverse) for the packed path, spread over R blocks of one row each
// in FP64: T = I - A X (A's upper triangle read), then X += X T.  On one SM
// the two R^3 products took ~1.2 ms at R = 128 (GB300 retires ~1.6 FP64
// FMA per clock per SM); this form runs them on R SMs.  T: R^2 doubles.
__global__ void newton_residual_kernel(int R, const double* __restrict__ A, const double* __restrict__ X,
                                       double* __restrict__ T) {
    __shared__ double arow[kMaxRank];
    const int i = blockIdx.x;
    for (int k = threadIdx.x; k < R; k += blockDim.x) arow[k] = i <= k ? A[i * R + k] : A[k * R + i];
    __syncthreads();
    for (int j = threadIdx.x; j < R; j += blockDim.x) {
        double acc = 0.0;
        for (int k = 0; k < R; k++) acc = fma(arow[k], X[k * R + j], acc);
        T[i * R + j] = (i == j ? 1.0 : 0.0) - acc;
    }
}
__global__ void newton_update_kernel(int R, const double* __restrict__ T, double* __restrict__ X) {
    __shared__ double xrow[kMaxRank];
    const int i = blockIdx.x;
    for (int k = threadIdx.x; k < R; k += blockDim.x) xrow[k] = X[i * R + k];
    __syncthreads();
    for (int j = threadIdx.x; j < R; j += blockDim.x) {
        double acc = 0.0;
        for (int k = 0; k < R; k++) acc = fma(xrow[k], T[k * R + j], acc);
        X[i * R + j] = xrow[j] + acc;
    }
}

// Shared memory of the Cholesky path (L, L^{-1}, and the Newton step's
// third matrix).  The Cholesky path in full matrices is used when its buffers
// fit under kPinvSmemCap (R <= 92); larger ranks take the packed kernel.
static size_t chol_smem_bytes(int R) { return sizeof(double) * 3 * (size_t)R * R; }
static size_t chol_packed_smem_bytes(int R) { return sizeof(double) * 2 * (size_t)(R * (R + 1) / 2); }
constexpr size_t kPinvSmemCap = 200 * 1024;

size_t pinv_smem_bytes(int R) {
    size_t jac = syev_smem_bytes(R);
    if (chol_smem_bytes(R) > kPinvSmemCap) return jac;
    return std::max(chol_smem_bytes(R), jac);
}

static int launch_pinv_impl(int R, const double* A, double* out, double tol, double* vt_scratch, int refine,
                            cudaStream_t stream) {
    if (R <= kSmallPinvMaxR) {
        const size_t smem = std::max(syev_smem_bytes(R), chol_smem_bytes(R));
        spd_pinv_small_kernel<<<1, kSmallPinvThreads, smem, stream>>>(R, A, out, tol, vt_scratch, refine);
        count_launch();
        EXAFAC_CHECK_LAUNCH();
        return EXAFAC_OK;
    }
    const int fast = chol_smem_bytes(R) <= kPinvSmemCap;
    if (!fast) {
        const size_t smem = std::max(chol_packed_smem_bytes(R), syev_smem_bytes(R));
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(spd_pinv_packed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        spd_pinv_packed_kernel<<<1, 512, smem, stream>>>(R, A, out, tol, vt_scratch, 0);
        count_launch();
        if (refine) {
            newton_residual_kernel<<<R, 128, 0, stream>>>(R, A, out, vt_scratch);
            count_launch();
            newton_update_kernel<<<R, 128, 0, stream>>>(R, vt_scratch, out);
            count_launch();
        }
        EXAFAC_CHECK_LAUNCH();
        return EXAFAC_OK;
    }
    size_t smem = pinv_smem_bytes(R);
    if (smem > 48 * 1024)
        EXAFAC_CUDA_TRY(cudaFuncSetAttribute(spd_pinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    spd_pinv_kernel<<<1, R <= 32 ? 256 : 512, smem, stream>>>(R, A, out, tol, vt_scratch, fast ? refine : 0, fast);
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int launch_pinv(int R, const double* A, double* out, double tol, double* vt_scratch, cudaStream_t stream) {
    return launch_pinv_impl(R, A, out, tol, vt_scratch, 0, stream);
}

int launch_pinv_refined(int R, const double* A, double* out, double tol, double* vt_scratch, cudaStream_t stream) {
    return launch_pinv_impl(R, A, out, tol, vt_scratch, 1, stream);
}

int launch_sigma_pinv_f32(int R, const double* ugram, double* sigma, double* ngram, int* degenerate, double* out,
                          double tol, double* vt_scratch, cudaStream_t stream) {
    const size_t smem = std::max(syev_smem_bytes(R), chol_smem_bytes(R));
    EXAFAC_CUDA_TRY(launch_dependent(sigma_pinv_kernel, 1, kSmallPinvThreads, smem, stream, R, ugram, sigma, ngram,
                                     degenerate, out, tol, vt_scratch));
    count_launch();
    EXAFAC_CHECK_LAUNCH();
    return EXAFAC_OK;
}

int launch_pinv_leverage_f32(int R, const double* A, double* out, double tol, double* vt_scratch,
                             cudaStream_t stream) {
    if (R > kSmallPinvMaxR) return launch_pinv_impl(R, A, out, tol, vt_scratch, 0, stream);
    return launch_pinv_impl(R, A, out, tol, vt_scratch, 2, stream);
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

// ---------------------------------------------------------------------------
// STS-CP computeM of the mixed forms (sts_cp.hpp:80-188 with Cholesky factors
// in place of the two eigendecompositions).
//
// The draws use, per sampled mode, rows e_v with sum_v e_v e_v^T = M (the
// eigen tree picks v, then the row tree a row by (U_i . (h * e_v))^2): the
// row is then drawn with probability proportional to (h * U_i)^T M (h * U_i)
// whatever factor supplies the rows, so any E with E^T E = M gives the same
// distribution of rows and weights as the reference's scaled eigenvectors
// (only the intermediate leaf v differs).  The FP64 form keeps the
// eigenvectors, which reproduce the reference's draws; the mixed forms take
// Cholesky factors: about R^3 / 3 FP64 FMAs each, against some ten Jacobi
// sweeps of about 5 R^3.
//
// sts_phi_chol_kernel (one CTA): A = chain[first] (the Hadamard product of
// every Gram but mode n's) = L L^T, Phi = A^{-1} = L^{-T} L^{-1}, taken when
// lambda_min >= 1 / ||A^{-1}||_F > 10 tol (as the Cholesky pseudo-inverse
// above); the rows of L^{-1} are a factor of Phi and become E[N].  Otherwise
// the CTA computes the Jacobi eigendecomposition and the reference's
// W = V Lambda^{-1/2} (eigenvalues <= tol dropped).  Then chain[k] *= Phi
// for k >= 1, k != n.
//
// sts_chain_chol_kernel (one CTA per k = 1..N-1, k != n): the pivoted
// Cholesky P^T chain[k] P = L L^T (largest remaining diagonal first; stops
// once it is <= R eps times the largest diagonal, the rest of the matrix, a
// positive semidefinite remainder with entries that small, dropped): E[k]
// row v = column v of P L.
// ---------------------------------------------------------------------------

// Right-looking Cholesky of the packed lower triangle L (tri(i, j), j <= i),
// in place.  piv != nullptr: symmetric pivoting on the largest remaining
// diagonal (piv[j] = the original index at position j), stopping when it is
// <= stop; *rank = the number of columns factored.  piv == nullptr: stops at
// a pivot that is not a positive finite number, *rank = its position.
// col: R doubles of shared scratch.  Every thread returns the same *rank.
__device__ void chol_packed_block(int R, double* L, int* piv, double stop, double* col, int* rank) {
    __shared__ int s_p;
    __shared__ int s_stop;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (piv)
        for (int i = tid; i < R; i += nt) piv[i] = i;
    if (tid == 0) s_stop = R;
    __syncthreads();
    for (int k = 0; k < R; k++) {
        if (piv) {
            if (tid < 32) {  // warp 0: the largest remaining diagonal (first index on ties)
                double best = -1.0;
                int bi = k;
                for (int i = k + tid; i < R; i += 32) {
                    const double d = L[tri(i, i)];
                    if (d > best) {
                        best = d;
                        bi = i;
                    }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    const double ob = __shfl_down_sync(0xffffffffu, best, o);
                    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) {
                        best = ob;
                        bi = oi;
                    }
                }
                if (tid == 0) {
                    s_p = bi;
                    if (!(best > stop)) s_stop = k;
                }
            }
            __syncthreads();
            if (s_stop == k) break;
            const int p = s_p;
            if (p != k) {  // swap rows and columns k and p (disjoint element pairs)
                for (int j = tid; j < R; j += nt) {
                    double *x = nullptr, *y = nullptr;
                    if (j < k) {
                        x = &L[tri(k, j)];
                        y = &L[tri(p, j)];
                    } else if (j == k) {
                        x = &L[tri(k, k)];
                        y = &L[tri(p, p)];
                    } else if (j < p) {
                        x = &L[tri(j, k)];
                        y = &L[tri(p, j)];
                    } else if (j > p) {
                        x = &L[tri(j, k)];
                        y = &L[tri(j, p)];
                    }
                    if (x) {
                        const double t = *x;
                        *x = *y;
                        *y = t;
                    }
                }
                if (tid == 0) {
                    const int t = piv[k];
                    piv[k] = piv[p];
                    piv[p] = t;
                }
            }
            __syncthreads();
        } else {
            const double d = L[tri(k, k)];
            if (!(d > 0.0) || !isfinite(d)) {  // the same in every thread
                if (tid == 0) s_stop = k;
                break;
            }
        }
        const double lkk = sqrt(L[tri(k, k)]);
        for (int i = k + 1 + tid; i < R; i += nt) col[i] = L[tri(i, k)] / lkk;
        __syncthreads();
        if (tid == 0) L[tri(k, k)] = lkk;
        {  // the trailing lower triangle: a warp per row, its lanes along the row
            const int wid = tid >> 5, lane = tid & 31, nw = nt >> 5;
            for (int i = k + 1 + wid; i < R; i += nw) {
                const double ci = col[i];
                double* row = L + tri(i, 0);
                for (int j = k + 1 + lane; j < i; j += 32) row[j] -= ci * col[j];
                if (lane == 0) {
                    row[i] -= ci * ci;
                    row[k] = ci;
                }
            }
        }
        __syncthreads();
    }
    __syncthreads();
    *rank = s_stop;
}

__global__ void sts_phi_chol_kernel(int N, int n, int R, int first, double tol, double* __restrict__ chain,
                                    double* __restrict__ E, double* __restrict__ Phi, double* __restrict__ PhiP,
                                    double* __restrict__ V, double* __restrict__ lam, double* __restrict__ vt) {
    extern __shared__ double smem[];
    __shared__ double fro_w[32];
    __shared__ double col[kMaxRank];
    const int P = R * (R + 1) / 2, R2 = R * R;
    const int tid = threadIdx.x, nt = blockDim.x;
    double* L = smem;
    double* Li = smem + P;
    const double* A = chain + (int64_t)first * R2;
    double* EN = E + (int64_t)N * R2;
    for (int i = tid >> 5; i < R; i += nt >> 5)  // a warp per row of the packed lower triangle
        for (int j = tid & 31; j <= i; j += 32) {
            L[tri(i, j)] = A[j * R + i];  // upper triangle of A
            Li[tri(i, j)] = 0.0;
        }
    __syncthreads();
    int rank;
    chol_packed_block(R, L, nullptr, 0.0, col, &rank);
    bool ok = rank == R;
    if (ok) {
        for (int c = tid; c < R; c += nt) {  // L^{-1}, column c by forward substitution
            for (int i = c; i < R; i++) {
                const double s = sub_dot(L, Li, i, c, c, i, (i == c) ? 1.0 : 0.0);
                Li[tri(i, c)] = s / L[tri(i, i)];
            }
        }
        __syncthreads();
        double part = 0.0;
        for (int e = tid; e < R2; e += nt) {  // Phi = L^{-T} L^{-1}: (a, b), a <= b, once and mirrored
            const int a = e / R, b = e % R;
            if (a > b) continue;
            const double acc = gram_dot(Li, a, b, b, R);
            Phi[a * R + b] = acc;
            Phi[b * R + a] = acc;
            part += (a == b ? 1.0 : 2.0) * (acc * acc);
        }
        part = warp_sum(part);
        if ((tid & 31) == 0) fro_w[tid >> 5] = part;
        __syncthreads();
        double fro = 0.0;
        for (int q = 0; q < (nt + 31) / 32; q++) fro += fro_w[q];
        ok = isfinite(fro) && 1.0 / sqrt(fro) > 10.0 * tol;  // the same in every thread
        if (ok)
            for (int e = tid; e < R2; e += nt) {  // E[N] row v = row v of L^{-1}
                const int v = e / R, u = e % R;
                EN[e] = u <= v ? Li[tri(v, u)] : 0.0;
            }
    }
    __syncthreads();
    if (!ok) {  // Jacobi: W[:, R-1-v] = eigenvector v / sqrt(lambda_v), lambda_v > tol
        syev_block(R, A, V, lam, nullptr, tol, vt, smem);
        __syncthreads();
        for (int e = tid; e < R2; e += nt) {
            const int a = e / R, b = e % R;
            const int v = R - 1 - a;
            EN[e] = lam[v] > tol ? V[b * R + v] / sqrt(lam[v]) : 0.0;
        }
        __syncthreads();
        for (int e = tid; e < R2; e += nt) {
            const int a = e / R, b = e % R;
            double acc = 0.0;
            for (int w = 0; w < R; w++) acc = fma(EN[w * R + a], EN[w * R + b], acc);
            Phi[e] = acc;
        }
    }
    __syncthreads();
    for (int e = tid; e < R2; e += nt) {
        const int a = e / R, b = e % R;
        const double p = Phi[a <= b ? a * R + b : b * R + a];
        if (a <= b) PhiP[a * R - a * (a - 1) / 2 + (b - a)] = p;  // packed upper triangle, rows in order
        for (int k = N - 1; k > 0; k--)
            if (k != n) chain[(int64_t)k * R2 + e] *= p;
    }
}

__global__ void sts_chain_chol_kernel(int N, int n, int R, const double* __restrict__ chain, double* __restrict__ E) {
    extern __shared__ double smem[];
    __shared__ double col[kMaxRank];
    __shared__ int piv[kMaxRank];
    __shared__ double dmax_w[32];
    const int k = blockIdx.x;
    if (k == 0 || k == n || k >= N) return;
    const int R2 = R * R;
    const int tid = threadIdx.x, nt = blockDim.x;
    const double* A = chain + (int64_t)k * R2;
    double* Ek = E + (int64_t)k * R2;
    double* L = smem;
    for (int i = tid >> 5; i < R; i += nt >> 5)  // a warp per row of the packed lower triangle
        for (int j = tid & 31; j <= i; j += 32) L[tri(i, j)] = A[j * R + i];
    double dm = 0.0;
    for (int i = tid; i < R; i += nt) dm = fmax(dm, A[i * R + i]);
    for (int o = 16; o > 0; o >>= 1) dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
    if ((tid & 31) == 0) dmax_w[tid >> 5] = dm;
    __syncthreads();
    double dmax = 0.0;
    for (int q = 0; q < (nt + 31) / 32; q++) dmax = fmax(dmax, dmax_w[q]);
    int rank;
    chol_packed_block(R, L, piv, (double)R * 2.220446049250313e-16 * dmax, col, &rank);
    for (int e = tid; e < R2; e += nt) {  // E[k][v][piv[i]] = L[i][v]
        const int v = e / R, i = e % R;
        Ek[v * R + piv[i]] = (v < rank && i >= v) ? L[tri(i, v)] : 0.0;
    }
}

size_t sts_factor_smem_bytes(int R) {
    return std::max(sizeof(double) * 2 * (size_t)(R * (R + 1) / 2), syev_smem_bytes(R));
}

int launch_sts_factors_chol(int N, int n, int R, double tol, double* chain, double* E, double* Phi, double* PhiP,
                            double* V, double* lam, double* vt, cudaStream_t stream) {
    const size_t smem = sts_factor_smem_bytes(R);
    EXAFAC_CUDA_TRY(cudaFuncSetAttribute(sts_phi_chol_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int first = (n == 0) ? 1 : 0;
    sts_phi_chol_kernel<<<1, 512, smem, stream>>>(N, n, R, first, tol, chain, E, Phi, PhiP, V, lam, vt);
    count_launch();
    const size_t fsm = sizeof(double) * (size_t)(R * (R + 1) / 2);
    if (fsm > 48 * 1024)
        EXAFAC_CUDA_TRY(
            cudaFuncSetAttribute(sts_chain_chol_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm));
    if (N > 1) {
        sts_chain_chol_kernel<<<N, 512, fsm, stream>>>(N, n, R, chain, E);
        count_launch();
    }
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
    return launch_pinv(R, A, out, tol, (double*)workspace, (cudaStream_t)stream);
}
