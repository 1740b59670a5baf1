// trsm.cuh -- device-pointer triangular solves.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// Column-major TRSM (cblas semantics, cblas enum values), device pointers.
void dev_dtrsm(int side, int uplo, int ta, int diag, int M, int N, double alpha, const double *A, int lda,
               double *B, int ldb, cudaStream_t st);
void dev_strsm(int side, int uplo, int ta, int diag, int M, int N, float alpha, const float *A, int lda, float *B,
               int ldb, cudaStream_t st);
// L11 * X = B with L11 = unit lower A[k:k+n, k:k+n] (n <= 64): the LU's U12 solve.
void dev_trsm_llnu_block(const double *A, int lda, int k, int n, double *B, int ldb, int ncols, cudaStream_t st);
void dev_trsm_llnu_block(const float *A, int lda, int k, int n, float *B, int ldb, int ncols, cudaStream_t st);

}  // namespace atlg
