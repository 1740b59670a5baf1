/* Level-1 routines the extracted tester programs and test-library routines
 * call; tester_glue.c binds them to the reference BLAS (asum, copy) or
 * implements them (zero, gecopy).  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_TESTER_LEVEL1_H
#define REFSHIM_TESTER_LEVEL1_H
#include "atlas_misc.h"
double ATL_dasum(const int N, const double *X, const int incX);
float  ATL_sasum(const int N, const float *X, const int incX);
void ATL_dcopy(const int N, const double *X, const int incX, double *Y, const int incY);
void ATL_scopy(const int N, const float *X, const int incX, float *Y, const int incY);
void ATL_dzero(const int N, double *X, const int incX);
void ATL_szero(const int N, float *X, const int incX);
void ATL_dgecopy(const int M, const int N, const double *A, const int lda, double *C, const int ldc);
void ATL_sgecopy(const int M, const int N, const float *A, const int lda, float *C, const int ldc);
#endif
