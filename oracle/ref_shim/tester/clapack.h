/* clapack prototypes (the reference's C LAPACK interface) called by the
 * extracted LU tester; resolved by the library under test.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_CLAPACK_H
#define REFSHIM_CLAPACK_H
#include "cblas.h"
int clapack_dgetrf(const enum CBLAS_ORDER Order, const int M, const int N, double *A,
                   const int lda, int *ipiv);
int clapack_sgetrf(const enum CBLAS_ORDER Order, const int M, const int N, float *A,
                   const int lda, int *ipiv);
#endif
