// Small dense FP64 R x R kernels (eigendecomposition, pseudo-inverse).
#pragma once
#include "common.cuh"

namespace exafac {

size_t syev_smem_bytes(int R);
size_t syev_scratch_doubles(int R, int batch);

// Batched symmetric eigendecomposition / pseudo-inverse, one CTA per matrix
// (matrix b at A + b * a_stride, upper triangle read).  V, lam, pinv may be
// null.  vt_scratch: syev_scratch_doubles(R, batch) doubles.
int launch_syev(int R, const double* A, int64_t a_stride, int batch, double* V, double* lam, int64_t v_stride,
                double* pinv, double tol, double* vt_scratch, cudaStream_t stream);

// Symmetric pseudo-inverse (eigenvalues <= tol dropped) of one matrix:
// Cholesky inverse when provably well conditioned, Jacobi otherwise.
int launch_pinv(int R, const double* A, double* out, double tol, double* vt_scratch, cudaStream_t stream);

// The same followed by one Newton step X <- 2X - X A X (the refinement the
// mixed forms apply to the solve).  For R > 92 the step runs in vt_scratch,
// which must then hold 2 R^2 doubles.
int launch_pinv_refined(int R, const double* A, double* out, double tol, double* vt_scratch, cudaStream_t stream);
// The leverage-score pseudo-inverse of the mixed forms (unit-diagonal Gram):
// the sweep in FP32 when its error bound allows, else the FP64 path.
// R <= 32: sigma, ngram and the degenerate flag from the factor Gram, then
// the FP32-first leverage pseudo-inverse of ngram, in one launch.
int launch_sigma_pinv_f32(int R, const double* ugram, double* sigma, double* ngram, int* degenerate, double* out,
                          double tol, double* vt_scratch, cudaStream_t stream);
int launch_pinv_leverage_f32(int R, const double* A, double* out, double tol, double* vt_scratch,
                             cudaStream_t stream);

// STS-CP computeM of the mixed forms from Cholesky factors: Phi (full and
// packed), E[N] and chain[k] *= Phi from chain[first] (Jacobi when not
// provably well conditioned; V, lam, vt its scratch), then E[k] for k = 1..
// N-1, k != n, from the pivoted Cholesky of chain[k].
int launch_sts_factors_chol(int N, int n, int R, double tol, double* chain, double* E, double* Phi, double* PhiP,
                            double* V, double* lam, double* vt, cudaStream_t stream);

}  // namespace exafac
