// getri.cuh -- device-pointer triangular inverse and inverse from LU factors.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// ATL_trtri semantics (Order, Uplo, Diag); 0 or the 1-based index of the
// first zero on a non-unit diagonal.  Synchronizes once (the zero check).
int dev_dtrtri(int order, int uplo, int diag, int n, double *A, int lda, cudaStream_t st);
int dev_strtri(int order, int uplo, int diag, int n, float *A, int lda, cudaStream_t st);
// Inverse of the matrix whose getrf factors (either order: the computation
// on the memory is the same) are in A, with 0-based pivots in host memory.
int dev_dgetri(int n, double *A, int lda, const int *ipiv_host, cudaStream_t st);
int dev_sgetri(int n, float *A, int lda, const int *ipiv_host, cudaStream_t st);

}  // namespace atlg
