// trmm.cuh -- device-pointer triangular matrix multiply.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// Column-major B = alpha*op(A)*B (side kLeft) or alpha*B*op(A) (kRight).
void dev_dtrmm(int side, int uplo, int ta, int diag, int M, int N, double alpha, const double *A, int lda,
               double *B, int ldb, cudaStream_t st);
void dev_strmm(int side, int uplo, int ta, int diag, int M, int N, float alpha, const float *A, int lda, float *B,
               int ldb, cudaStream_t st);

}  // namespace atlg
