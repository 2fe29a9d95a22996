// LAPACKE declaration for the reference build (oracle/_ref), resolved against
// scipy's bundled OpenBLAS.  Test infrastructure only.
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

int scipy_LAPACKE_dsyev(int matrix_layout, char jobz, char uplo, int n, double* a, int lda, double* w);

#ifdef __cplusplus
}
#endif

#define LAPACKE_dsyev scipy_LAPACKE_dsyev
