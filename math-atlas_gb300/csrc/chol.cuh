// chol.cuh -- device-pointer SYRK and Cholesky factorization / solve.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// C = alpha op(A) op(A)^T + beta C on the uplo triangle (trans: NoTrans -> A A^T, else A^T A).
void dev_dsyrk(int uplo, int trans, int n, int k, double alpha, const double *A, int lda, double beta, double *C,
               int ldc, cudaStream_t st);
void dev_ssyrk(int uplo, int trans, int n, int k, float alpha, const float *A, int lda, float beta, float *C,
               int ldc, cudaStream_t st);
// Lower triangle := transpose of the strict upper triangle.
void dev_dsyreflect(int n, double *C, int ldc, cudaStream_t st);
void dev_ssyreflect(int n, float *C, int ldc, cudaStream_t st);
// Column-major Cholesky of the uplo triangle; returns 0 or the 1-based index
// of the first non-positive pivot (synchronizes once per 64-column block).
int dev_dpotrf(int uplo, int n, double *A, int lda, cudaStream_t st);
int dev_spotrf(int uplo, int n, float *A, int lda, cudaStream_t st);
// ATL_potrs semantics (Order, Uplo) on device data.
void dev_dpotrs(int order, int uplo, int n, int nrhs, const double *A, int lda, double *B, int ldb, cudaStream_t st);
void dev_spotrs(int order, int uplo, int n, int nrhs, const float *A, int lda, float *B, int ldb, cudaStream_t st);

}  // namespace atlg
