// trmm.cu -- B = alpha*op(A)*B or alpha*B*op(A) with A triangular (cblas_?trmm)
// on GB300, FP64 and FP32, column-major.
//
// Reference interface replaced: the TRMM template of AtlasBase/Clint/
// cblas.base:587-692 (argument checks and the RowMajor flip of Side and
// Uplo, shared with TRSM) over ATL_trmm.
//
// GB300 design: one launch of the register-tiled GEMM in its triangular-
// operand mode.  B is first copied to a workspace W (device to device); then
// B = alpha*op(A)*W (Left) or alpha*W*op(A) (Right), where the GEMM reads
// op(A) through its triangle: k-tiles wholly outside the triangle are never
// loaded, the tiles that cross the diagonal are masked in shared memory (1 on
// a unit diagonal).  Half the flops of the dense product, one pass over B.
#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "trmm.cuh"

namespace atlg {

template <typename T>
static void trmm_impl(int side, int uplo, int ta, int diag, int M, int N, T alpha, const T *A, int lda, T *B,
                      int ldb, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  if (alpha == T(0)) {
    dev_gescal(M, N, T(0), B, ldb, st);
    return;
  }
  const int tA = (ta == kNoTrans) ? kNoTrans : kTrans;
  const bool opup = (uplo == kUpper) == (tA == kNoTrans);
  // workspace copy of B, leading dimension even so the GEMM can use TMA
  const int ldw = (M + 1) & ~1;
  T *W = static_cast<T *>(ctx().buffer(kBufTrmm, sizeof(T) * (size_t)ldw * N));
  ATLG_CHECK(cudaMemcpy2DAsync(W, sizeof(T) * ldw, B, sizeof(T) * ldb, sizeof(T) * M, N, cudaMemcpyDeviceToDevice,
                               st));
  GemmOpts o;
  o.tri = (side == kLeft ? kTriA : kTriB) | (opup ? kTriUpper : 0) | (diag == kUnit ? kTriUnit : 0);
  if (side == kLeft) {
    if (sizeof(T) == 8)
      dev_dgemm(tA, kNoTrans, M, N, M, (double)alpha, (const double *)A, lda, (const double *)W, ldw, 0.0,
                (double *)B, ldb, st, o);
    else
      dev_sgemm(tA, kNoTrans, M, N, M, (float)alpha, (const float *)A, lda, (const float *)W, ldw, 0.0f,
                (float *)B, ldb, st, o);
  } else {
    if (sizeof(T) == 8)
      dev_dgemm(kNoTrans, tA, M, N, N, (double)alpha, (const double *)W, ldw, (const double *)A, lda, 0.0,
                (double *)B, ldb, st, o);
    else
      dev_sgemm(kNoTrans, tA, M, N, N, (float)alpha, (const float *)W, ldw, (const float *)A, lda, 0.0f,
                (float *)B, ldb, st, o);
  }
}

void dev_dtrmm(int side, int uplo, int ta, int diag, int M, int N, double alpha, const double *A, int lda,
               double *B, int ldb, cudaStream_t st) {
  trmm_impl<double>(side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb, st);
}
void dev_strmm(int side, int uplo, int ta, int diag, int M, int N, float alpha, const float *A, int lda, float *B,
               int ldb, cudaStream_t st) {
  trmm_impl<float>(side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb, st);
}

}  // namespace atlg
