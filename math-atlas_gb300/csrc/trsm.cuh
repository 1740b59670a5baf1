// trsm.cuh -- device-pointer triangular solves.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// Column-major TRSM (cblas semantics, cblas enum values), device pointers.
void dev_dtrsm(int side, int uplo, int ta, int diag, int M, int N, double alpha, const double *A, int lda,
               double *B, int ldb, cudaStream_t st);
void dev_strsm(int side, int uplo, int ta, int diag, int M, int N, float alpha, const float *A, int lda, float *B,
               int ldb, cudaStream_t st);
// Left-side op(A) X = B (alpha 1, column-major) through 64 x 64 diagonal-block
// inverses formed once per call: for many right-hand sides (rounding differs
// from substitution).
void dev_dtrsm_left_inv(int uplo, int ta, int diag, int M, int N, const double *A, int lda, double *B, int ldb,
                        cudaStream_t st);
void dev_strsm_left_inv(int uplo, int ta, int diag, int M, int N, const float *A, int lda, float *B, int ldb,
                        cudaStream_t st);
// L11 * X = B with L11 = unit lower A[k:k+n, k:k+n] (n <= 64): the LU's U12 solve.
void dev_trsm_llnu_block(const double *A, int lda, int k, int n, double *B, int ldb, int ncols, cudaStream_t st);
void dev_trsm_llnu_block(const float *A, int lda, int k, int n, float *B, int ldb, int ncols, cudaStream_t st);

// op(A) x = x for one right-hand side, one launch (look-back over 64-row blocks).
void dev_dtrsv(int uplo, int ta, int diag, int n, const double *A, int lda, double *x, cudaStream_t st);
void dev_strsv(int uplo, int ta, int diag, int n, const float *A, int lda, float *x, cudaStream_t st);
// dev_strsv whose 64 x 64 diagonal blocks are applied as inverses formed
// while each block waits (for the mixed solver's FP32 refinement solves;
// rounding differs from substitution)
void dev_strsv_inv(int uplo, int ta, int diag, int n, const float *A, int lda, float *x, cudaStream_t st);
// Chained FP32 TRSV for one triangle solved many times (op(A) = A, one
// right-hand side): dev_strsv_chain_prepare forms the 128 x 128 diagonal-block
// inverses and couplings into ws (strsv_chain_ws_floats(n) floats) once per
// factorization; dev_strsv_chain solves with them (rounding differs from
// substitution).
size_t strsv_chain_ws_floats(int n);
void dev_strsv_chain_prepare(int uplo, int diag, int n, const float *A, int lda, float *ws, cudaStream_t st);
void dev_strsv_chain(int uplo, int n, const float *A, int lda, const float *ws, float *x, cudaStream_t st);
unsigned trsv_status_read_and_clear();

}  // namespace atlg
