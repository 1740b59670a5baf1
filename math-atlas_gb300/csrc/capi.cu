// capi.cu -- the drop-in C ABI: cblas_* / clapack_* with the reference's
// prototypes, argument checks, error messages and return conventions, plus
// device-pointer variants (atlg_*_dev) for callers whose data already lives
// in GPU memory.
//
// Host-pointer entry points are synchronous like the reference's: they copy
// the operands to cached device buffers (packed, leading dimension rounded
// up to an even count so TMA can address them), run on the library's stream
// and copy the results back before returning.
//
// Argument checking follows AtlasBase/Clint/cblas.base (cblas_errprn :14,
// cblas_xerbla :42 -- message to stderr and exit(-1); GEMM checks :119-216,
// TRSM/TRMM checks :611-677, SYRK :356-449), AtlasBase/Clint/cblas-lvl2.base
// (GEMV :21-93, TRSV :273-357) and AtlasBase/Clint/atlas-clp.base
// (clapack_gesv :62, clapack_getrf :140, clapack_getrs :218, clapack_posv
// :266, clapack_potrf :320, clapack_potrs :363, clapack_getri :115,
// clapack_trtri :411).
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/atlas_gb300.h"
#include "common.cuh"
#include "context.cuh"
#include "chol.cuh"
#include "gemm.cuh"
#include "getri.cuh"
#include "iamax.cuh"
#include "lu.cuh"
#include "lu_split.cuh"
#include "mixed.cuh"
#include "split.cuh"
#include "tf32.cuh"
#include "trmm.cuh"
#include "trsm.cuh"

using namespace atlg;

namespace atlg {
double probe_fp64_tflops();
double probe_fp32_tflops();
void probe_fp64_mma_tflops(double *m8n8k4, double *m16n8k4, double *m16n8k16);
}

// ------------------------------------------------------------ error reporting
extern "C" int cblas_errprn(int ierr, int info, const char *form, ...) {
  va_list ap;
  va_start(ap, form);
  vfprintf(stderr, form, ap);
  va_end(ap);
  return ierr < info ? ierr : info;
}

extern "C" void cblas_xerbla(int p, const char *rout, const char *form, ...) {
  va_list ap;
  va_start(ap, form);
  if (p) fprintf(stderr, "Parameter %d to routine %s was incorrect\n", p, rout);
  vfprintf(stderr, form, ap);
  va_end(ap);
  fflush(stderr);
  exit(-1);
}

namespace {

void check_status(const char *rout) {
  const unsigned s = gemm_status_read_and_clear() | lu_status_read_and_clear() | split_status_read_and_clear() |
                     tf32_status_read_and_clear() | trsv_status_read_and_clear();
  if (s) {
    fprintf(stderr, "atlas_gb300: %s: device wait gave up (status 0x%x)\n", rout, s);
    fflush(stderr);
    abort();
  }
}

inline int even_up(int n) { return n < 2 ? 2 : (n + 1) & ~1; }

template <typename T>
T *to_dev(int slot, const T *h, int rows, int cols, int ldh, int *ldd, cudaStream_t st) {
  *ldd = even_up(rows);
  T *d = static_cast<T *>(ctx().buffer(slot, sizeof(T) * (size_t)(*ldd) * (cols > 0 ? cols : 1)));
  if (rows > 0 && cols > 0)
    ATLG_CHECK(cudaMemcpy2DAsync(d, sizeof(T) * (*ldd), h, sizeof(T) * ldh, sizeof(T) * rows, cols,
                                 cudaMemcpyHostToDevice, st));
  return d;
}

template <typename T>
void to_host(T *h, int ldh, const T *d, int ldd, int rows, int cols, cudaStream_t st) {
  if (rows > 0 && cols > 0)
    ATLG_CHECK(cudaMemcpy2DAsync(h, sizeof(T) * ldh, d, sizeof(T) * ldd, sizeof(T) * rows, cols,
                                 cudaMemcpyDeviceToHost, st));
}


template <typename T>
void dev_syrk_any(int uplo, int trans, int n, int k, T alpha, const T *A, int lda, T beta, T *C, int ldc,
                  cudaStream_t st);

// ---------------------------------------------------------------------- GEMM
template <typename T>
int gemm_check(const char *rout, int Order, int TA, int TB, int M, int N, int K, int lda, int ldb, int ldc) {
  int info = 2000;
  if (M < 0) info = cblas_errprn(4, info, "M cannot be less than zero 0,; is set to %d.", M);
  if (N < 0) info = cblas_errprn(5, info, "N cannot be less than zero 0,; is set to %d.", N);
  if (K < 0) info = cblas_errprn(6, info, "K cannot be less than zero 0,; is set to %d.", K);
  if (Order == CblasRowMajor) {
    if (TA == CblasNoTrans) {
      if (lda < K || lda < 1) info = cblas_errprn(9, info, "lda must be >= MAX(K,1): lda=%d K=%d", lda, K);
    } else {
      if (TA != CblasConjTrans && TA != CblasTrans)
        info = cblas_errprn(2, info, "TransA must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                            CblasConjTrans, TA);
      if (lda < M || lda < 1) info = cblas_errprn(9, info, "lda must be >= MAX(M,1): lda=%d M=%d", lda, M);
    }
    if (TB == CblasNoTrans) {
      if (ldb < N || ldb < 1) info = cblas_errprn(11, info, "ldb must be >= MAX(N,1): ldb=%d N=%d", ldb, N);
    } else {
      if (TB != CblasConjTrans && TB != CblasTrans)
        info = cblas_errprn(3, info, "TransB must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                            CblasConjTrans, TB);
      if (ldb < K || ldb < 1) info = cblas_errprn(11, info, "ldb must be >= MAX(K,1): ldb=%d K=%d", ldb, K);
    }
    if (ldc < N || ldc < 1) info = cblas_errprn(14, info, "ldc must be >= MAX(N,1): ldc=%d N=%d", ldc, N);
  } else if (Order == CblasColMajor) {
    if (TA == CblasNoTrans) {
      if (lda < M || lda < 1) info = cblas_errprn(9, info, "lda must be >= MAX(M,1): lda=%d M=%d", lda, M);
    } else {
      if (TA != CblasConjTrans && TA != CblasTrans)
        info = cblas_errprn(2, info, "TransA must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                            CblasConjTrans, TA);
      if (lda < K || lda < 1) info = cblas_errprn(9, info, "lda must be >= MAX(K,1): lda=%d K=%d", lda, K);
    }
    if (TB == CblasNoTrans) {
      if (ldb < K || ldb < 1) info = cblas_errprn(11, info, "ldb must be >= MAX(K,1): ldb=%d K=%d", ldb, K);
    } else {
      if (TB != CblasConjTrans && TB != CblasTrans)
        info = cblas_errprn(3, info, "TransB must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                            CblasConjTrans, TB);
      if (ldb < N || ldb < 1) info = cblas_errprn(11, info, "ldb must be >= MAX(N,1): ldb=%d N=%d", ldb, N);
    }
    if (ldc < M || ldc < 1) info = cblas_errprn(14, info, "ldc must be >= MAX(M,1): ldc=%d M=%d", ldc, M);
  } else {
    info = cblas_errprn(1, info, "Order must be %d or %d, but is set to %d", CblasRowMajor, CblasColMajor, Order);
  }
  if (info != 2000) {
    cblas_xerbla(info, rout, "");
    return info;
  }
  return 0;
}

template <typename T>
void dev_gemm_any(int TA, int TB, int M, int N, int K, T alpha, const T *A, int lda, const T *B, int ldb, T beta,
                  T *C, int ldc, cudaStream_t st);
template <>
void dev_gemm_any<double>(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda,
                          const double *B, int ldb, double beta, double *C, int ldc, cudaStream_t st) {
  dev_dgemm(TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st);
}
template <>
void dev_gemm_any<float>(int TA, int TB, int M, int N, int K, float alpha, const float *A, int lda, const float *B,
                         int ldb, float beta, float *C, int ldc, cudaStream_t st) {
  dev_sgemm(TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st);
}

template <typename T>
void host_gemm(const char *rout, int Order, int TA, int TB, int M, int N, int K, T alpha, const T *A, int lda,
               const T *B, int ldb, T beta, T *C, int ldc) {
  if (gemm_check<T>(rout, Order, TA, TB, M, N, K, lda, ldb, ldc)) return;
  if (M == 0 || N == 0) return;
  // A op(A)^T asked for as a GEMM: SYRK of the upper triangle, then mirror
  // it (AtlasBase/Clint/cblas.base:220-231).  One operand must be NoTrans:
  // Trans against ConjTrans is A^T A^T for real data, not a SYRK.
  if (A == B && M == N && TA != TB && lda == ldb && beta == T(0) && K > 0 && alpha != T(0) &&
      (TA == CblasNoTrans || TB == CblasNoTrans)) {
    const int tr = (Order == CblasColMajor) ? TA : TB;
    cudaStream_t st = ctx().stream;
    int ldd_a, ldd_c = even_up(N);
    const T *dA = (tr == CblasNoTrans) ? to_dev<T>(kBufA, A, N, K, lda, &ldd_a, st)
                                       : to_dev<T>(kBufA, A, K, N, lda, &ldd_a, st);
    T *dC = static_cast<T *>(ctx().buffer(kBufC, sizeof(T) * (size_t)ldd_c * N));
    dev_syrk_any<T>(kUpper, tr == CblasNoTrans ? kNoTrans : kTrans, N, K, alpha, dA, ldd_a, beta, dC, ldd_c, st);
    if (sizeof(T) == 8) dev_dsyreflect(N, (double *)dC, ldd_c, st);
    else dev_ssyreflect(N, (float *)dC, ldd_c, st);
    to_host<T>(C, ldc, dC, ldd_c, N, N, st);
    ATLG_CHECK(cudaStreamSynchronize(st));
    check_status(rout);
    return;
  }
  if (Order == CblasRowMajor) {   // C^T = op(B)^T op(A)^T in column-major terms
    const T *t = A; A = B; B = t;
    int ti = lda; lda = ldb; ldb = ti;
    ti = TA; TA = TB; TB = ti;
    ti = M; M = N; N = ti;
  }
  cudaStream_t st = ctx().stream;
  int ldd_c;
  const bool need_c = (beta != T(0));
  T *dC;
  if (need_c) dC = to_dev<T>(kBufC, C, M, N, ldc, &ldd_c, st);
  else {
    ldd_c = even_up(M);
    dC = static_cast<T *>(ctx().buffer(kBufC, sizeof(T) * (size_t)ldd_c * N));
  }
  if (alpha != T(0) && K > 0) {
    const int ra = (TA == CblasNoTrans) ? M : K, ca = (TA == CblasNoTrans) ? K : M;
    const int rb = (TB == CblasNoTrans) ? K : N, cb = (TB == CblasNoTrans) ? N : K;
    int ldd_a, ldd_b;
    const T *dA = to_dev<T>(kBufA, A, ra, ca, lda, &ldd_a, st);
    const T *dB = to_dev<T>(kBufB, B, rb, cb, ldb, &ldd_b, st);
    dev_gemm_any<T>(TA, TB, M, N, K, alpha, dA, ldd_a, dB, ldd_b, beta, dC, ldd_c, st);
  } else {
    dev_gescal(M, N, beta, dC, ldd_c, st);
  }
  to_host<T>(C, ldc, dC, ldd_c, M, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
}

// ---------------------------------------------------------------------- TRSM
int trsm_check(const char *rout, int Order, int Side, int Uplo, int TA, int Diag, int M, int N, int lda, int ldb) {
  int info = 2000;
  if (Order == CblasColMajor) {
    if (Side == CblasLeft) {
      if (lda < M || lda < 1) info = cblas_errprn(10, info, "lda must be >= MAX(M,1): lda=%d M=%d", lda, M);
    } else if (Side == CblasRight) {
      if (lda < N || lda < 1) info = cblas_errprn(10, info, "lda must be >= MAX(N,1): lda=%d N=%d", lda, N);
    } else
      info = cblas_errprn(2, info, "SIDE must be %d or %d, but is set to %d", CblasRight, CblasLeft, Side);
    if (ldb < M || ldb < 1) info = cblas_errprn(12, info, "ldb must be >= MAX(M,1): ldb=%d M=%d", ldb, M);
  } else if (Order == CblasRowMajor) {
    if (Side == CblasLeft) {
      if (lda < M || lda < 1) info = cblas_errprn(10, info, "lda must be >= MAX(M,1): lda=%d M=%d", lda, M);
    } else if (Side == CblasRight) {
      if (lda < N || lda < 1) info = cblas_errprn(10, info, "lda must be >= MAX(N,1): lda=%d N=%d", lda, N);
    } else
      info = cblas_errprn(2, info, "SIDE must be %d or %d, but is set to %d", CblasRight, CblasLeft, Side);
    if (ldb < N || ldb < 1) info = cblas_errprn(12, info, "ldb must be >= MAX(N,1): ldb=%d N=%d", ldb, N);
  } else
    info = cblas_errprn(1, info, "Order must be %d or %d, but is set to %d", CblasRowMajor, CblasColMajor, Order);
  if (Uplo != CblasUpper && Uplo != CblasLower)
    info = cblas_errprn(3, info, "UPLO must be %d or %d, but is set to %d", CblasUpper, CblasLower, Uplo);
  if (TA != CblasNoTrans && TA != CblasTrans && TA != CblasConjTrans)
    info = cblas_errprn(4, info, "TransA must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                        CblasConjTrans, TA);
  if (Diag != CblasUnit && Diag != CblasNonUnit)
    info = cblas_errprn(5, info, "UPLO must be %d or %d, but is set to %d", CblasUnit, CblasNonUnit, Diag);
  if (M < 0) info = cblas_errprn(6, info, "M cannot be less than zero; it is set to %d.", M);
  if (N < 0) info = cblas_errprn(7, info, "N cannot be less than zero; it is set to %d.", N);
  if (info != 2000) {
    cblas_xerbla(info, rout, "");
    return info;
  }
  return 0;
}

template <typename T>
void dev_trsm_any(int side, int uplo, int ta, int diag, int M, int N, T alpha, const T *A, int lda, T *B, int ldb,
                  cudaStream_t st) {
  if (sizeof(T) == 8)
    dev_dtrsm(side, uplo, ta, diag, M, N, (double)alpha, (const double *)A, lda, (double *)B, ldb, st);
  else
    dev_strsm(side, uplo, ta, diag, M, N, (float)alpha, (const float *)A, lda, (float *)B, ldb, st);
}

template <typename T>
void host_trsm(const char *rout, int Order, int Side, int Uplo, int TA, int Diag, int M, int N, T alpha, const T *A,
               int lda, T *B, int ldb) {
  if (trsm_check(rout, Order, Side, Uplo, TA, Diag, M, N, lda, ldb)) return;
  if (Order == CblasRowMajor) {
    Side = (Side == CblasLeft) ? CblasRight : CblasLeft;
    Uplo = (Uplo == CblasUpper) ? CblasLower : CblasUpper;
    const int t = M; M = N; N = t;
  }
  if (M == 0 || N == 0) return;
  cudaStream_t st = ctx().stream;
  const int na = (Side == CblasLeft) ? M : N;
  int ldd_a, ldd_b;
  const T *dA = to_dev<T>(kBufA, A, na, na, lda, &ldd_a, st);
  T *dB = to_dev<T>(kBufB, B, M, N, ldb, &ldd_b, st);
  dev_trsm_any<T>(Side, Uplo, TA, Diag, M, N, alpha, dA, ldd_a, dB, ldd_b, st);
  to_host<T>(B, ldb, dB, ldd_b, M, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
}

// ---------------------------------------------------------------- LAPACK LU
template <typename T>
void dev_getrf_any(int M, int N, T *A, int lda, int *ipiv, int *info, cudaStream_t st) {
  if (sizeof(T) == 8) dev_dgetrf(M, N, (double *)A, lda, ipiv, info, st);
  else dev_sgetrf(M, N, (float *)A, lda, ipiv, info, st);
}
template <typename T>
void dev_getrs_any(int order, int trans, int N, int NRHS, const T *A, int lda, const int *ipiv, T *B, int ldb,
                   cudaStream_t st) {
  if (sizeof(T) == 8) dev_dgetrs(order, trans, N, NRHS, (const double *)A, lda, ipiv, (double *)B, ldb, st);
  else dev_sgetrs(order, trans, N, NRHS, (const float *)A, lda, ipiv, (float *)B, ldb, st);
}

// getrf on host data; the factor stays on the device (kBufA, ld *ldd) for gesv.
template <typename T>
int host_getrf_keep(int Order, int M, int N, T *A, int lda, int *ipiv, T **dA_out, int *ldd_out, int **dpiv_out) {
  cudaStream_t st = ctx().stream;
  // RowMajor M x N is the column-major N x M matrix; ATL_getrfR is the
  // column-pivoted LU of it, i.e. the row-pivoted LU of the transpose.
  const int rows = (Order == CblasColMajor) ? M : N, cols = (Order == CblasColMajor) ? N : M;
  const int MN = M < N ? M : N;
  int ldd;
  T *dA = to_dev<T>(kBufA, A, rows, cols, lda, &ldd, st);
  int *dpiv = static_cast<int *>(ctx().buffer(kBufPiv, sizeof(int) * (size_t)(MN > 0 ? MN : 1)));
  int *dinfo = static_cast<int *>(ctx().buffer(kBufInfo, sizeof(int) * 4));
  dev_getrf_any<T>(rows, cols, dA, ldd, dpiv, dinfo, st);
  int info = 0;
  to_host<T>(A, lda, dA, ldd, rows, cols, st);
  if (MN > 0) ATLG_CHECK(cudaMemcpyAsync(ipiv, dpiv, sizeof(int) * MN, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  if (dA_out) *dA_out = dA;
  if (ldd_out) *ldd_out = ldd;
  if (dpiv_out) *dpiv_out = dpiv;
  return info;
}

template <typename T>
int host_getrf(const char *rout, int Order, int M, int N, T *A, int lda, int *ipiv) {
  if (Order != CblasRowMajor && Order != CblasColMajor)
    cblas_xerbla(1, rout, "Order must be %d or %d, but is set to %d\n", CblasRowMajor, CblasColMajor, Order);
  if (M < 0) cblas_xerbla(2, rout, "M cannot be less than zero 0,; is set to %d.\n", M);
  if (N < 0) cblas_xerbla(3, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (Order == CblasColMajor) {
    if (lda < M || lda < 1) cblas_xerbla(6, rout, "lda must be >= MAX(M,1): lda=%d M=%d\n", lda, M);
  } else {
    if (lda < N || lda < 1) cblas_xerbla(6, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  }
  if (M == 0 || N == 0) return 0;
  const int info = host_getrf_keep<T>(Order, M, N, A, lda, ipiv, nullptr, nullptr, nullptr);
  check_status(rout);
  return info;
}

template <typename T>
int host_getrs(const char *rout, int Order, int Trans, int N, int NRHS, const T *A, int lda, const int *ipiv, T *B,
               int ldb) {
  if (Order != CblasRowMajor && Order != CblasColMajor)
    cblas_xerbla(1, rout, "Order must be %d or %d, but is set to %d\n", CblasRowMajor, CblasColMajor, Order);
  if (Trans != CblasNoTrans && Trans != CblasTrans && Trans != CblasConjTrans)
    cblas_xerbla(2, rout, "Trans must be %d, %d, or %d, but is set to %d\n", CblasNoTrans, CblasTrans,
                 CblasConjTrans, Trans);
  if (N < 0) cblas_xerbla(3, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (NRHS < 0) cblas_xerbla(4, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", NRHS);
  if (lda < N || lda < 1) cblas_xerbla(6, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (ldb < N || ldb < 1) cblas_xerbla(9, rout, "ldb must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (N == 0 || NRHS == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd_a, ldd_b;
  const T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd_a, st);
  int *dpiv = static_cast<int *>(ctx().buffer(kBufPiv, sizeof(int) * (size_t)N));
  ATLG_CHECK(cudaMemcpyAsync(dpiv, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, st));
  T *dB = to_dev<T>(kBufB, B, N, NRHS, ldb, &ldd_b, st);
  dev_getrs_any<T>(Order, Trans, N, NRHS, dA, ldd_a, dpiv, dB, ldd_b, st);
  to_host<T>(B, ldb, dB, ldd_b, N, NRHS, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return 0;
}

template <typename T>
int host_gesv(const char *rout, int Order, int N, int NRHS, T *A, int lda, int *ipiv, T *B, int ldb) {
  if (Order != CblasRowMajor && Order != CblasColMajor)
    cblas_xerbla(1, rout, "Order must be %d or %d, but is set to %d.\n", CblasRowMajor, CblasColMajor, Order);
  if (N < 0) cblas_xerbla(2, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (NRHS < 0) cblas_xerbla(3, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", NRHS);
  if (lda < N || lda < 1) cblas_xerbla(5, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (ldb < N || ldb < 1) cblas_xerbla(8, rout, "ldb must be >= MAX(N,1): ldb=%d N=%d\n", ldb, N);
  if (N == 0) return 0;
  // A and B up, the factorization, then at once the solve on the library
  // stream while the factors, pivots and info go back on a second stream;
  // the solution is copied back only when info is 0 (a singular A leaves B
  // as it was, as in the reference; the solve that ran anyway is dropped).
  Context &c = ctx();
  cudaStream_t st = c.stream, cs = c.outer_stream();
  int ldd_a, ldd_b = 0;
  T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd_a, st);
  T *dB = NRHS > 0 ? to_dev<T>(kBufB, B, N, NRHS, ldb, &ldd_b, st) : nullptr;
  int *dpiv = static_cast<int *>(c.buffer(kBufPiv, sizeof(int) * (size_t)N));
  int *dinfo = static_cast<int *>(c.buffer(kBufInfo, sizeof(int) * 4));
  dev_getrf_any<T>(N, N, dA, ldd_a, dpiv, dinfo, st);
  cudaEvent_t ev = c.sync_event(5);
  ATLG_CHECK(cudaEventRecord(ev, st));
  if (NRHS > 0) dev_getrs_any<T>(Order, CblasNoTrans, N, NRHS, dA, ldd_a, dpiv, dB, ldd_b, st);
  ATLG_CHECK(cudaStreamWaitEvent(cs, ev, 0));
  int info = 0;
  ATLG_CHECK(cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, cs));
  ATLG_CHECK(cudaMemcpyAsync(ipiv, dpiv, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost, cs));
  to_host<T>(A, lda, dA, ldd_a, N, N, cs);
  ATLG_CHECK(cudaStreamSynchronize(cs));
  if (info == 0 && NRHS > 0) to_host<T>(B, ldb, dB, ldd_b, N, NRHS, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

// ------------------------------------------------------- SYRK and Cholesky
// cblas_?syrk: checks and the RowMajor flip of Uplo and Trans follow
// AtlasBase/Clint/cblas.base:356-449.
int syrk_check(const char *rout, int Order, int Uplo, int Trans, int N, int K, int lda, int ldc) {
  int info = 2000;
  if (Uplo != CblasUpper && Uplo != CblasLower)
    info = cblas_errprn(2, info, "UPLO must be %d or %d, but is set to %d", CblasUpper, CblasLower, Uplo);
  if (N < 0) info = cblas_errprn(4, info, "N cannot be less than zero; it is set to %d.", N);
  if (K < 0) info = cblas_errprn(5, info, "K cannot be less than zero; it is set to %d.", K);
  if (Order == CblasColMajor || Order == CblasRowMajor) {
    // ColMajor NoTrans and RowMajor Trans store A with N rows per column
    const bool n_rows = (Order == CblasColMajor) == (Trans == CblasNoTrans);
    if (Trans != CblasNoTrans && Trans != CblasTrans && Trans != CblasConjTrans)
      info = cblas_errprn(3, info, "Trans must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                          CblasConjTrans, Trans);
    if (n_rows) {
      if (lda < N || lda < 1) info = cblas_errprn(8, info, "lda must be >= MAX(N,1): lda=%d N=%d", lda, N);
    } else {
      if (lda < K || lda < 1) info = cblas_errprn(8, info, "lda must be >= MAX(K,1): lda=%d K=%d", lda, K);
    }
  } else
    info = cblas_errprn(1, info, "Order must be %d or %d, but is set to %d", CblasRowMajor, CblasColMajor, Order);
  if (ldc < N || ldc < 1) info = cblas_errprn(11, info, "ldc must be >= MAX(N,1): ldc=%d N=%d", ldc, N);
  if (info != 2000) {
    cblas_xerbla(info, rout, "");
    return info;
  }
  return 0;
}

template <typename T>
void dev_syrk_any(int uplo, int trans, int n, int k, T alpha, const T *A, int lda, T beta, T *C, int ldc,
                  cudaStream_t st) {
  if (sizeof(T) == 8)
    dev_dsyrk(uplo, trans, n, k, (double)alpha, (const double *)A, lda, (double)beta, (double *)C, ldc, st);
  else
    dev_ssyrk(uplo, trans, n, k, (float)alpha, (const float *)A, lda, (float)beta, (float *)C, ldc, st);
}

template <typename T>
void host_syrk(const char *rout, int Order, int Uplo, int Trans, int N, int K, T alpha, const T *A, int lda, T beta,
               T *C, int ldc) {
  if (syrk_check(rout, Order, Uplo, Trans, N, K, lda, ldc)) return;
  if (Order == CblasRowMajor) {
    Uplo = (Uplo == CblasUpper) ? CblasLower : CblasUpper;
    Trans = (Trans == CblasNoTrans) ? CblasTrans : CblasNoTrans;
  }
  if (N == 0) return;
  if (Trans == CblasConjTrans) Trans = CblasTrans;
  cudaStream_t st = ctx().stream;
  int ldd_a = 2, ldd_c;
  // the whole square goes both ways, so the other triangle comes back as it was
  T *dC = to_dev<T>(kBufC, C, N, N, ldc, &ldd_c, st);
  const T *dA = nullptr;
  if (K > 0 && alpha != T(0))
    dA = (Trans == CblasNoTrans) ? to_dev<T>(kBufA, A, N, K, lda, &ldd_a, st) : to_dev<T>(kBufA, A, K, N, lda, &ldd_a, st);
  dev_syrk_any<T>(Uplo, Trans, N, K, alpha, dA, ldd_a, beta, dC, ldd_c, st);
  to_host<T>(C, ldc, dC, ldd_c, N, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
}

template <typename T>
int dev_potrf_any(int uplo, int n, T *A, int lda, cudaStream_t st) {
  return (sizeof(T) == 8) ? dev_dpotrf(uplo, n, (double *)A, lda, st) : dev_spotrf(uplo, n, (float *)A, lda, st);
}
template <typename T>
void dev_potrs_any(int order, int uplo, int n, int nrhs, const T *A, int lda, T *B, int ldb, cudaStream_t st) {
  if (sizeof(T) == 8) dev_dpotrs(order, uplo, n, nrhs, (const double *)A, lda, (double *)B, ldb, st);
  else dev_spotrs(order, uplo, n, nrhs, (const float *)A, lda, (float *)B, ldb, st);
}

// ATL_potrf's dispatch (AtlasBase/Clint/atlas-lp.base:336-357): RowMajor
// real data is the column-major factorization of the other triangle.
inline int potrf_uplo(int Order, int Uplo) {
  const int u = (Uplo == CblasUpper) ? kUpper : kLower;
  if (Order == CblasColMajor) return u;
  return u == kUpper ? kLower : kUpper;
}

// clapack_?potrf / ?potrs / ?posv argument checks (AtlasBase/Clint/
// atlas-clp.base:266-410).  Unlike cblas, every failing check calls xerbla.
void lp_check_ou(const char *rout, int Order, int Uplo, int N) {
  if (Order != CblasRowMajor && Order != CblasColMajor)
    cblas_xerbla(1, rout, "Order must be %d or %d, but is set to %d\n", CblasRowMajor, CblasColMajor, Order);
  if (Uplo != CblasUpper && Uplo != CblasLower)
    cblas_xerbla(2, rout, "Uplo must be %d or %d, but is set to %d\n", CblasUpper, CblasLower, Uplo);
  if (N < 0) cblas_xerbla(3, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
}

template <typename T>
int host_potrf(const char *rout, int Order, int Uplo, int N, T *A, int lda) {
  lp_check_ou(rout, Order, Uplo, N);
  if (lda < N || lda < 1) cblas_xerbla(5, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (N == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd;
  T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd, st);
  const int info = dev_potrf_any<T>(potrf_uplo(Order, Uplo), N, dA, ldd, st);
  to_host<T>(A, lda, dA, ldd, N, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

template <typename T>
int host_potrs(const char *rout, int Order, int Uplo, int N, int NRHS, const T *A, int lda, T *B, int ldb) {
  lp_check_ou(rout, Order, Uplo, N);
  if (NRHS < 0) cblas_xerbla(4, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", NRHS);
  if (lda < N || lda < 1) cblas_xerbla(6, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (ldb < N || ldb < 1) cblas_xerbla(8, rout, "ldb must be >= MAX(N,1): ldb=%d N=%d\n", ldb, N);
  if (N == 0 || NRHS == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd_a, ldd_b;
  const T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd_a, st);
  T *dB = to_dev<T>(kBufB, B, N, NRHS, ldb, &ldd_b, st);
  dev_potrs_any<T>(Order, Uplo == CblasUpper ? kUpper : kLower, N, NRHS, dA, ldd_a, dB, ldd_b, st);
  to_host<T>(B, ldb, dB, ldd_b, N, NRHS, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return 0;
}

template <typename T>
int host_posv(const char *rout, int Order, int Uplo, int N, int NRHS, T *A, int lda, T *B, int ldb) {
  lp_check_ou(rout, Order, Uplo, N);
  if (NRHS < 0) cblas_xerbla(4, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", NRHS);
  if (lda < N || lda < 1) cblas_xerbla(6, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (ldb < N || ldb < 1) cblas_xerbla(8, rout, "ldb must be >= MAX(N,1): ldb=%d N=%d\n", ldb, N);
  if (N == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd_a;
  T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd_a, st);
  const int info = dev_potrf_any<T>(potrf_uplo(Order, Uplo), N, dA, ldd_a, st);
  to_host<T>(A, lda, dA, ldd_a, N, N, st);
  if (info == 0 && NRHS > 0) {
    int ldd_b;
    T *dB = to_dev<T>(kBufB, B, N, NRHS, ldb, &ldd_b, st);
    dev_potrs_any<T>(Order, Uplo == CblasUpper ? kUpper : kLower, N, NRHS, dA, ldd_a, dB, ldd_b, st);
    to_host<T>(B, ldb, dB, ldd_b, N, NRHS, st);
  }
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

// ---------------------------------------------------------------- TRMM
template <typename T>
void dev_trmm_any(int side, int uplo, int ta, int diag, int M, int N, T alpha, const T *A, int lda, T *B, int ldb,
                  cudaStream_t st) {
  if (sizeof(T) == 8)
    dev_dtrmm(side, uplo, ta, diag, M, N, (double)alpha, (const double *)A, lda, (double *)B, ldb, st);
  else
    dev_strmm(side, uplo, ta, diag, M, N, (float)alpha, (const float *)A, lda, (float *)B, ldb, st);
}

// cblas_?trmm: TRSM's checks and RowMajor flip (AtlasBase/Clint/cblas.base:587-692).
template <typename T>
void host_trmm(const char *rout, int Order, int Side, int Uplo, int TA, int Diag, int M, int N, T alpha, const T *A,
               int lda, T *B, int ldb) {
  if (trsm_check(rout, Order, Side, Uplo, TA, Diag, M, N, lda, ldb)) return;
  if (Order == CblasRowMajor) {
    Side = (Side == CblasLeft) ? CblasRight : CblasLeft;
    Uplo = (Uplo == CblasUpper) ? CblasLower : CblasUpper;
    const int t = M; M = N; N = t;
  }
  if (M == 0 || N == 0) return;
  cudaStream_t st = ctx().stream;
  const int na = (Side == CblasLeft) ? M : N;
  int ldd_a, ldd_b;
  const T *dA = to_dev<T>(kBufA, A, na, na, lda, &ldd_a, st);
  T *dB = to_dev<T>(kBufB, B, M, N, ldb, &ldd_b, st);
  dev_trmm_any<T>(Side, Uplo, TA, Diag, M, N, alpha, dA, ldd_a, dB, ldd_b, st);
  to_host<T>(B, ldb, dB, ldd_b, M, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
}

// ------------------------------------------------------------ GEMV, TRSV
// Strided host vector <-> contiguous copy; a negative increment counts from
// the far end, as the cblas wrappers arrange (AtlasBase/Clint/cblas-lvl2.base:
// 71-80, 339).
template <typename T>
void vec_pack(std::vector<T> &v, const T *X, int n, int inc) {
  v.resize(n > 0 ? n : 1);
  for (int i = 0; i < n; ++i) v[i] = X[inc > 0 ? (size_t)i * inc : (size_t)(n - 1 - i) * (size_t)(-inc)];
}
template <typename T>
void vec_unpack(const std::vector<T> &v, T *X, int n, int inc) {
  for (int i = 0; i < n; ++i) X[inc > 0 ? (size_t)i * inc : (size_t)(n - 1 - i) * (size_t)(-inc)] = v[i];
}

// cblas_i?amax (AtlasBase/Clint/cblas-lvl1.base:408-420): ATL_i?amax when
// N > 0 and incX > 0, else 0; ATL_i?amax itself returns 0 for N < 2.  A
// strided vector is packed on the host and searched with the strided form's
// final rule (no zero-magnitude check, atlas-lvl1.base:1318-1340).
template <typename T>
int host_iamax(int N, const T *X, int incX) {
  if (N < 2 || incX <= 0) return 0;
  cudaStream_t st = ctx().stream;
  std::vector<T> hx;
  const T *src = X;
  if (incX != 1) {
    vec_pack(hx, X, N, incX);
    src = hx.data();
  }
  T *dx = static_cast<T *>(ctx().buffer(kBufB, sizeof(T) * (size_t)N));
  int *dres = static_cast<int *>(ctx().buffer(kBufInfo, sizeof(int)));
  ATLG_CHECK(cudaMemcpyAsync(dx, src, sizeof(T) * (size_t)N, cudaMemcpyHostToDevice, st));
  if (sizeof(T) == 8) dev_idamax(N, (const double *)dx, 1, incX == 1, dres, st);
  else dev_isamax(N, (const float *)dx, 1, incX == 1, dres, st);
  int res = 0;
  ATLG_CHECK(cudaMemcpyAsync(&res, dres, sizeof(int), cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  return res;
}

template <typename T>
int iamax_dev(int N, const T *X, int incX, int *result, void *stream) {
  if (N < 0) return -1;
  cudaStream_t st = stream_of(stream);
  if (N < 2 || incX <= 0) {
    ATLG_CHECK(cudaMemsetAsync(result, 0, sizeof(int), st));
    return 0;
  }
  if (sizeof(T) == 8) dev_idamax(N, (const double *)X, incX, incX == 1, result, st);
  else dev_isamax(N, (const float *)X, incX, incX == 1, result, st);
  return 0;
}

template <typename T>
void host_gemv(const char *rout, int Order, int TA, int M, int N, T alpha, const T *A, int lda, const T *X, int incX,
               T beta, T *Y, int incY) {
  int info = 2000;
  if (TA != CblasNoTrans && TA != CblasTrans && TA != CblasConjTrans)
    info = cblas_errprn(2, info, "TransA must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                        CblasConjTrans, TA);
  if (M < 0) info = cblas_errprn(3, info, "M cannot be less than zero; is set to %d.", M);
  if (N < 0) info = cblas_errprn(4, info, "N cannot be less than zero; is set to %d.", N);
  if (!incX) info = cblas_errprn(9, info, "incX cannot be zero; is set to %d.", incX);
  if (!incY) info = cblas_errprn(12, info, "incY cannot be zero; is set to %d.", incY);
  if (Order == CblasColMajor) {
    if (lda < M || lda < 1) info = cblas_errprn(7, info, "lda must be >= MAX(M,1): lda=%d M=%d", lda, M);
  } else if (Order == CblasRowMajor) {
    if (lda < N || lda < 1) info = cblas_errprn(7, info, "lda must be >= MAX(N,1): lda=%d N=%d", lda, N);
  } else
    info = cblas_errprn(1, info, "Order must be %d or %d, but is set to %d", CblasRowMajor, CblasColMajor, Order);
  if (info != 2000) {
    cblas_xerbla(info, rout, "");
    return;
  }
  if (M == 0 || N == 0) return;
  const int lx = (TA == CblasNoTrans) ? N : M, ly = (TA == CblasNoTrans) ? M : N;
  // column-major view: A has ra x ca entries; op is TA (ColMajor) or its flip
  const int ra = (Order == CblasColMajor) ? M : N, ca = (Order == CblasColMajor) ? N : M;
  int op = (TA == CblasNoTrans) ? kNoTrans : kTrans;
  if (Order == CblasRowMajor) op = (op == kNoTrans) ? kTrans : kNoTrans;
  cudaStream_t st = ctx().stream;
  std::vector<T> hx, hy;
  vec_pack(hx, X, lx, incX);
  if (beta != T(0)) vec_pack(hy, Y, ly, incY);
  else hy.assign(ly, T(0));
  int ldd_a;
  const T *dA = to_dev<T>(kBufA, A, ra, ca, lda, &ldd_a, st);
  T *dx = static_cast<T *>(ctx().buffer(kBufB, sizeof(T) * (size_t)lx));
  T *dy = static_cast<T *>(ctx().buffer(kBufC, sizeof(T) * (size_t)ly));
  ATLG_CHECK(cudaMemcpyAsync(dx, hx.data(), sizeof(T) * lx, cudaMemcpyHostToDevice, st));
  if (beta != T(0)) ATLG_CHECK(cudaMemcpyAsync(dy, hy.data(), sizeof(T) * ly, cudaMemcpyHostToDevice, st));
  if (sizeof(T) == 8)
    dev_dgemv(op, ly, lx, (double)alpha, (const double *)dA, ldd_a, (const double *)dx, 1, (double)beta,
              (double *)dy, st);
  else
    dev_sgemv(op, ly, lx, (float)alpha, (const float *)dA, ldd_a, (const float *)dx, 1, (float)beta, (float *)dy,
              st);
  ATLG_CHECK(cudaMemcpyAsync(hy.data(), dy, sizeof(T) * ly, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  vec_unpack(hy, Y, ly, incY);
  check_status(rout);
}

template <typename T>
void host_trsv(const char *rout, int Order, int Uplo, int TA, int Diag, int N, const T *A, int lda, T *X, int incX) {
  int info = 2000;
  if (Order != CblasColMajor && Order != CblasRowMajor)
    info = cblas_errprn(1, info, "Order must be %d or %d, but is set to %d", CblasRowMajor, CblasColMajor, Order);
  if (Uplo != CblasUpper && Uplo != CblasLower)
    info = cblas_errprn(2, info, "UPLO must be %d or %d, but is set to %d", CblasUpper, CblasLower, Uplo);
  if (TA != CblasNoTrans && TA != CblasTrans && TA != CblasConjTrans)
    info = cblas_errprn(3, info, "TransA must be %d, %d or %d, but is set to %d", CblasNoTrans, CblasTrans,
                        CblasConjTrans, TA);
  if (Diag != CblasUnit && Diag != CblasNonUnit)
    info = cblas_errprn(4, info, "DIAG must be %d or %d, but is set to %d", CblasUnit, CblasNonUnit, Diag);
  if (N < 0) info = cblas_errprn(5, info, "N cannot be less than zero; is set to %d.", N);
  if (lda < N || lda < 1) info = cblas_errprn(7, info, "lda must be >= MAX(N,1): lda=%d N=%d", lda, N);
  if (!incX) info = cblas_errprn(9, info, "incX cannot be zero; is set to %d.", incX);
  if (info != 2000) {
    cblas_xerbla(info, rout, "");
    return;
  }
  if (N == 0) return;
  int uplo = (Uplo == CblasUpper) ? kUpper : kLower;
  int ta = (TA == CblasNoTrans) ? kNoTrans : kTrans;
  if (Order == CblasRowMajor) {
    uplo = (uplo == kUpper) ? kLower : kUpper;
    ta = (ta == kNoTrans) ? kTrans : kNoTrans;
  }
  cudaStream_t st = ctx().stream;
  std::vector<T> hx;
  vec_pack(hx, X, N, incX);
  int ldd_a;
  const T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd_a, st);
  T *dx = static_cast<T *>(ctx().buffer(kBufB, sizeof(T) * (size_t)N));
  ATLG_CHECK(cudaMemcpyAsync(dx, hx.data(), sizeof(T) * N, cudaMemcpyHostToDevice, st));
  if (sizeof(T) == 8) dev_dtrsv(uplo, ta, Diag, N, (const double *)dA, ldd_a, (double *)dx, st);
  else dev_strsv(uplo, ta, Diag, N, (const float *)dA, ldd_a, (float *)dx, st);
  ATLG_CHECK(cudaMemcpyAsync(hx.data(), dx, sizeof(T) * N, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  vec_unpack(hx, X, N, incX);
  check_status(rout);
}

// ------------------------------------------------------------ inverses
// clapack_?trtri (AtlasBase/Clint/atlas-clp.base:411-452).  The reference
// tests `if (ierr)` on an uninitialised ierr before calling ATL_trtri; the
// inverse is computed here whenever the arguments are valid.
template <typename T>
int host_trtri(const char *rout, int Order, int Uplo, int Diag, int N, T *A, int lda) {
  if (Order != CblasRowMajor && Order != CblasColMajor)
    cblas_xerbla(1, rout, "Order must be %d or %d, but is set to %d\n", CblasRowMajor, CblasColMajor, Order);
  if (Uplo != CblasUpper && Uplo != CblasLower)
    cblas_xerbla(2, rout, "Uplo must be %d or %d, but is set to %d\n", CblasUpper, CblasLower, Uplo);
  if (Diag != CblasUnit && Diag != CblasNonUnit)
    cblas_xerbla(3, rout, "Diag must be %d or %d, but is set to %d\n", CblasNonUnit, CblasUnit, Diag);
  if (N < 0) cblas_xerbla(4, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (lda < N || lda < 1) cblas_xerbla(6, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (N == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd;
  T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd, st);
  const int info = (sizeof(T) == 8) ? dev_dtrtri(Order, Uplo, Diag, N, (double *)dA, ldd, st)
                                    : dev_strtri(Order, Uplo, Diag, N, (float *)dA, ldd, st);
  if (info == 0) to_host<T>(A, lda, dA, ldd, N, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

// clapack_?getri (AtlasBase/Clint/atlas-clp.base:115-139): the reference
// checks no argument; N < 0 and lda < max(N,1) are reported here through
// xerbla as parameters 2 and 4 instead of reading out of bounds.
template <typename T>
int host_getri(const char *rout, int Order, int N, T *A, int lda, const int *ipiv) {
  if (N < 0) cblas_xerbla(2, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (lda < N || lda < 1) cblas_xerbla(4, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  (void)Order;   // same computation on the same memory for both orders
  if (N == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd;
  T *dA = to_dev<T>(kBufA, A, N, N, lda, &ldd, st);
  const int info = (sizeof(T) == 8) ? dev_dgetri(N, (double *)dA, ldd, ipiv, st)
                                    : dev_sgetri(N, (float *)dA, ldd, ipiv, st);
  if (info == 0) to_host<T>(A, lda, dA, ldd, N, N, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

// ------------------------------------------------------------- new methods
int mixed_dev(int N, int NRHS, double *A, int lda, int *ipiv, const double *B, int ldb, double *X, int ldx,
              double *berr, double *ferr, int *iters, int *status, cudaStream_t st) {
  MixedResult r;
  const int info = dev_dgesv_mixed(N, NRHS, A, lda, ipiv, B, ldb, X, ldx, &r, st);
  for (int j = 0; j < NRHS; ++j) {
    if (berr) berr[j] = r.berr[j];
    if (ferr) ferr[j] = r.ferr[j];
  }
  if (iters) *iters = r.iters;
  if (status) *status = r.status;
  return info;
}

void adjoint_dev(int n, int nrhs, const double *LU, int lda, const int *ipiv, const double *X, int ldx,
                 const double *gX, int ldgx, double *gA, int ldga, double *gB, int ldgb, cudaStream_t st) {
  // gB = A^{-T} gX via the transposed solve on the stored factors (ATL_getrs
  // Trans: AtlasBase/Clint/atlas-lp.base:1675-1682), then gA = -gB X^T.
  ATLG_CHECK(cudaMemcpy2DAsync(gB, sizeof(double) * ldgb, gX, sizeof(double) * ldgx, sizeof(double) * n, nrhs,
                               cudaMemcpyDeviceToDevice, st));
  dev_dgetrs(kColMajor, kTrans, n, nrhs, LU, lda, ipiv, gB, ldgb, st);
  dev_dgemm(kNoTrans, kTrans, n, n, nrhs, -1.0, gB, ldgb, X, ldx, 0.0, gA, ldga, st);
}

}  // namespace

// ============================================================== C ABI: host
extern "C" {

void cblas_dgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const enum CBLAS_TRANSPOSE TB,
                 const int M, const int N, const int K, const double alpha, const double *A, const int lda,
                 const double *B, const int ldb, const double beta, double *C, const int ldc) {
  host_gemm<double>("cblas_dgemm", Order, TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}

void cblas_sgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const enum CBLAS_TRANSPOSE TB,
                 const int M, const int N, const int K, const float alpha, const float *A, const int lda,
                 const float *B, const int ldb, const float beta, float *C, const int ldc) {
  host_gemm<float>("cblas_sgemm", Order, TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}

void cblas_dtrsm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE TA, const enum CBLAS_DIAG Diag, const int M, const int N,
                 const double alpha, const double *A, const int lda, double *B, const int ldb) {
  host_trsm<double>("cblas_dtrsm", Order, Side, Uplo, TA, Diag, M, N, alpha, A, lda, B, ldb);
}

void cblas_strsm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE TA, const enum CBLAS_DIAG Diag, const int M, const int N,
                 const float alpha, const float *A, const int lda, float *B, const int ldb) {
  host_trsm<float>("cblas_strsm", Order, Side, Uplo, TA, Diag, M, N, alpha, A, lda, B, ldb);
}

int clapack_dgetrf(const enum CBLAS_ORDER Order, const int M, const int N, double *A, const int lda, int *ipiv) {
  return host_getrf<double>("clapack_dgetrf", Order, M, N, A, lda, ipiv);
}
int clapack_sgetrf(const enum CBLAS_ORDER Order, const int M, const int N, float *A, const int lda, int *ipiv) {
  return host_getrf<float>("clapack_sgetrf", Order, M, N, A, lda, ipiv);
}
int clapack_dgetrs(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE Trans, const int N, const int NRHS,
                   const double *A, const int lda, const int *ipiv, double *B, const int ldb) {
  return host_getrs<double>("clapack_dgetrs", Order, Trans, N, NRHS, A, lda, ipiv, B, ldb);
}
int clapack_sgetrs(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE Trans, const int N, const int NRHS,
                   const float *A, const int lda, const int *ipiv, float *B, const int ldb) {
  return host_getrs<float>("clapack_sgetrs", Order, Trans, N, NRHS, A, lda, ipiv, B, ldb);
}
int clapack_dgesv(const enum CBLAS_ORDER Order, const int N, const int NRHS, double *A, const int lda, int *ipiv,
                  double *B, const int ldb) {
  return host_gesv<double>("clapack_dgesv", Order, N, NRHS, A, lda, ipiv, B, ldb);
}
int clapack_sgesv(const enum CBLAS_ORDER Order, const int N, const int NRHS, float *A, const int lda, int *ipiv,
                  float *B, const int ldb) {
  return host_gesv<float>("clapack_sgesv", Order, N, NRHS, A, lda, ipiv, B, ldb);
}

void cblas_dsyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
                 const int N, const int K, const double alpha, const double *A, const int lda, const double beta,
                 double *C, const int ldc) {
  host_syrk<double>("cblas_dsyrk", Order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc);
}
void cblas_ssyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
                 const int N, const int K, const float alpha, const float *A, const int lda, const float beta,
                 float *C, const int ldc) {
  host_syrk<float>("cblas_ssyrk", Order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc);
}
int clapack_dpotrf(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N, double *A, const int lda) {
  return host_potrf<double>("clapack_dpotrf", Order, Uplo, N, A, lda);
}
int clapack_spotrf(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N, float *A, const int lda) {
  return host_potrf<float>("clapack_spotrf", Order, Uplo, N, A, lda);
}
int clapack_dpotrs(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const int N, const int NRHS,
                   const double *A, const int lda, double *B, const int ldb) {
  return host_potrs<double>("clapack_dpotrs", Order, Uplo, N, NRHS, A, lda, B, ldb);
}
int clapack_spotrs(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const int N, const int NRHS,
                   const float *A, const int lda, float *B, const int ldb) {
  return host_potrs<float>("clapack_spotrs", Order, Uplo, N, NRHS, A, lda, B, ldb);
}
int clapack_dposv(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N, const int NRHS, double *A,
                  const int lda, double *B, const int ldb) {
  return host_posv<double>("clapack_dposv", Order, Uplo, N, NRHS, A, lda, B, ldb);
}
int clapack_sposv(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N, const int NRHS, float *A,
                  const int lda, float *B, const int ldb) {
  return host_posv<float>("clapack_sposv", Order, Uplo, N, NRHS, A, lda, B, ldb);
}

void cblas_dtrmm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE TA, const enum CBLAS_DIAG Diag, const int M, const int N,
                 const double alpha, const double *A, const int lda, double *B, const int ldb) {
  host_trmm<double>("cblas_dtrmm", Order, Side, Uplo, TA, Diag, M, N, alpha, A, lda, B, ldb);
}
void cblas_strmm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE TA, const enum CBLAS_DIAG Diag, const int M, const int N,
                 const float alpha, const float *A, const int lda, float *B, const int ldb) {
  host_trmm<float>("cblas_strmm", Order, Side, Uplo, TA, Diag, M, N, alpha, A, lda, B, ldb);
}
int cblas_idamax(const int N, const double *X, const int incX) { return host_iamax<double>(N, X, incX); }
int cblas_isamax(const int N, const float *X, const int incX) { return host_iamax<float>(N, X, incX); }
void cblas_dgemv(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const int M, const int N,
                 const double alpha, const double *A, const int lda, const double *X, const int incX,
                 const double beta, double *Y, const int incY) {
  host_gemv<double>("cblas_dgemv", Order, TA, M, N, alpha, A, lda, X, incX, beta, Y, incY);
}
void cblas_sgemv(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const int M, const int N,
                 const float alpha, const float *A, const int lda, const float *X, const int incX,
                 const float beta, float *Y, const int incY) {
  host_gemv<float>("cblas_sgemv", Order, TA, M, N, alpha, A, lda, X, incX, beta, Y, incY);
}
void cblas_dtrsv(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_DIAG Diag, const int N, const double *A, const int lda, double *X,
                 const int incX) {
  host_trsv<double>("cblas_dtrsv", Order, Uplo, TA, Diag, N, A, lda, X, incX);
}
void cblas_strsv(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_DIAG Diag, const int N, const float *A, const int lda, float *X,
                 const int incX) {
  host_trsv<float>("cblas_strsv", Order, Uplo, TA, Diag, N, A, lda, X, incX);
}

int clapack_dtrtri(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const enum ATLAS_DIAG Diag,
                   const int N, double *A, const int lda) {
  return host_trtri<double>("clapack_dtrtri", Order, Uplo, Diag, N, A, lda);
}
int clapack_strtri(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const enum ATLAS_DIAG Diag,
                   const int N, float *A, const int lda) {
  return host_trtri<float>("clapack_strtri", Order, Uplo, Diag, N, A, lda);
}
int clapack_dgetri(const enum CBLAS_ORDER Order, const int N, double *A, const int lda, const int *ipiv) {
  return host_getri<double>("clapack_dgetri", Order, N, A, lda, ipiv);
}
int clapack_sgetri(const enum CBLAS_ORDER Order, const int N, float *A, const int lda, const int *ipiv) {
  return host_getri<float>("clapack_sgetri", Order, N, A, lda, ipiv);
}

// Split-DGEMM form of dgesv (no reference counterpart; see lu_split.cu):
// clapack_dgesv's ColMajor interface and checks; the LU's trailing updates run
// on the split-precision DGEMM with 8 slices, the solve is the FP64 getrs.
int dgesv_split(const int N, const int NRHS, double *A, const int lda, int *ipiv, double *B, const int ldb) {
  const char *rout = "dgesv_split";
  if (N < 0) cblas_xerbla(1, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (NRHS < 0) cblas_xerbla(2, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", NRHS);
  if (lda < N || lda < 1) cblas_xerbla(4, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (ldb < N || ldb < 1) cblas_xerbla(7, rout, "ldb must be >= MAX(N,1): ldb=%d N=%d\n", ldb, N);
  if (N == 0) return 0;
  cudaStream_t st = ctx().stream;
  int ldd;
  double *dA = to_dev<double>(kBufA, A, N, N, lda, &ldd, st);
  int *dpiv = static_cast<int *>(ctx().buffer(kBufPiv, sizeof(int) * (size_t)N));
  const int info = dev_dgetrf_split(N, dA, ldd, dpiv, 8, 1024, st);
  to_host<double>(A, lda, dA, ldd, N, N, st);
  ATLG_CHECK(cudaMemcpyAsync(ipiv, dpiv, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
  if (info == 0 && NRHS > 0) {
    int ldd_b;
    double *dB = to_dev<double>(kBufB, B, N, NRHS, ldb, &ldd_b, st);
    dev_dgetrs(kColMajor, kNoTrans, N, NRHS, dA, ldd, dpiv, dB, ldd_b, st);
    to_host<double>(B, ldb, dB, ldd_b, N, NRHS, st);
  }
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

// Split-precision DGEMM (no reference counterpart; see split.cu): the
// cblas_dgemm interface and checks, plus the number of 7-bit slices per
// operand (1..8; 7 gives about 49 bits of each row/column's largest entry).
void dgemm_split(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const enum CBLAS_TRANSPOSE TB,
                 const int M, const int N, const int K, const double alpha, const double *A, const int lda,
                 const double *B, const int ldb, const double beta, double *C, const int ldc, const int nslices) {
  const char *rout = "dgemm_split";
  if (gemm_check<double>(rout, Order, TA, TB, M, N, K, lda, ldb, ldc)) return;
  if (nslices < 1 || nslices > 8) cblas_xerbla(15, rout, "nslices must be in 1..8: %d\n", nslices);
  if (M == 0 || N == 0) return;
  int ta = TA, tb = TB, m = M, n = N, la = lda, lb = ldb;
  const double *a = A, *b = B;
  if (Order == CblasRowMajor) {
    a = B; b = A; la = ldb; lb = lda; ta = TB; tb = TA; m = N; n = M;
  }
  cudaStream_t st = ctx().stream;
  int ldd_c;
  double *dC;
  if (beta != 0.0) dC = to_dev<double>(kBufC, C, m, n, ldc, &ldd_c, st);
  else {
    ldd_c = even_up(m);
    dC = static_cast<double *>(ctx().buffer(kBufC, sizeof(double) * (size_t)ldd_c * n));
  }
  const int ra = (ta == CblasNoTrans) ? m : K, ca = (ta == CblasNoTrans) ? K : m;
  const int rb = (tb == CblasNoTrans) ? K : n, cb = (tb == CblasNoTrans) ? n : K;
  int ldd_a, ldd_b;
  const double *dA = to_dev<double>(kBufA, a, ra, ca, la, &ldd_a, st);
  const double *dB = to_dev<double>(kBufB, b, rb, cb, lb, &ldd_b, st);
  dev_dgemm_split(ta, tb, m, n, K, alpha, dA, ldd_a, dB, ldd_b, beta, dC, ldd_c, nslices, st);
  to_host<double>(C, ldc, dC, ldd_c, m, n, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
}

// Mixed-precision solve (no reference counterpart; see mixed.cu).  Column-
// major.  A is unchanged unless the FP64 fallback ran (status 1: A then
// holds the FP64 factors, as LAPACK dsgesv leaves them); B is unchanged; X
// gets the solution; berr/ferr have NRHS entries.  Returns 0, a negative
// argument index, or i > 0 when the FP64 factor has an exactly zero pivot.
int dgesv_mixed(const int N, const int NRHS, double *A, const int lda, int *ipiv, const double *B, const int ldb,
                double *X, const int ldx, double *berr, double *ferr, int *iters, int *status) {
  const char *rout = "dgesv_mixed";
  if (N < 0) cblas_xerbla(1, rout, "N cannot be less than zero 0,; is set to %d.\n", N);
  if (NRHS < 0) cblas_xerbla(2, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", NRHS);
  if (lda < N || lda < 1) cblas_xerbla(4, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, N);
  if (ldb < N || ldb < 1) cblas_xerbla(7, rout, "ldb must be >= MAX(N,1): ldb=%d N=%d\n", ldb, N);
  if (ldx < N || ldx < 1) cblas_xerbla(9, rout, "ldx must be >= MAX(N,1): ldx=%d N=%d\n", ldx, N);
  if (iters) *iters = 0;
  if (status) *status = 0;
  if (N == 0 || NRHS == 0) return 0;
  cudaStream_t st = ctx().stream;
  int lda_d, ldb_d, ldx_d;
  double *dA = to_dev<double>(kBufA, A, N, N, lda, &lda_d, st);
  const double *dB = to_dev<double>(kBufB, B, N, NRHS, ldb, &ldb_d, st);
  ldx_d = lda_d;
  double *dX = static_cast<double *>(ctx().buffer(kBufC, sizeof(double) * (size_t)ldx_d * NRHS));
  int *dpiv = static_cast<int *>(ctx().buffer(kBufPiv, sizeof(int) * (size_t)N));
  int st_out = 0;
  const int info = mixed_dev(N, NRHS, dA, lda_d, dpiv, dB, ldb_d, dX, ldx_d, berr, ferr, iters, &st_out, st);
  if (status) *status = st_out;
  to_host<double>(X, ldx, dX, ldx_d, N, NRHS, st);
  if (st_out != 0) to_host<double>(A, lda, dA, lda_d, N, N, st);
  ATLG_CHECK(cudaMemcpyAsync(ipiv, dpiv, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return info;
}

// Adjoint of X = A^{-1} B for an upstream gradient gX, on the stored
// factors (LU, ipiv) of clapack_dgetrf: gB = A^{-T} gX, gA = -gB X^T.
// No reference counterpart; the transposed solve is ATL_getrs Trans.
int dgesv_adjoint(const int n, const int nrhs, const double *LU, const int lda, const int *ipiv, const double *X,
                  const int ldx, const double *gX, const int ldgx, double *gA, const int ldga, double *gB,
                  const int ldgb) {
  const char *rout = "dgesv_adjoint";
  if (n < 0) cblas_xerbla(1, rout, "N cannot be less than zero 0,; is set to %d.\n", n);
  if (nrhs < 0) cblas_xerbla(2, rout, "NRHS cannot be less than zero 0,; is set to %d.\n", nrhs);
  if (lda < n || lda < 1) cblas_xerbla(4, rout, "lda must be >= MAX(N,1): lda=%d N=%d\n", lda, n);
  if (ldx < n || ldx < 1) cblas_xerbla(7, rout, "ldx must be >= MAX(N,1): ldx=%d N=%d\n", ldx, n);
  if (ldgx < n || ldgx < 1) cblas_xerbla(9, rout, "ldgx must be >= MAX(N,1): ldgx=%d N=%d\n", ldgx, n);
  if (ldga < n || ldga < 1) cblas_xerbla(11, rout, "ldga must be >= MAX(N,1): ldga=%d N=%d\n", ldga, n);
  if (ldgb < n || ldgb < 1) cblas_xerbla(13, rout, "ldgb must be >= MAX(N,1): ldgb=%d N=%d\n", ldgb, n);
  if (n == 0) return 0;
  cudaStream_t st = ctx().stream;
  int l_lu, l_x, l_gx;
  const double *dLU = to_dev<double>(kBufA, LU, n, n, lda, &l_lu, st);
  const double *dX = to_dev<double>(kBufB, X, n, nrhs, ldx, &l_x, st);
  const double *dgX = to_dev<double>(kBufW7, gX, n, nrhs, ldgx, &l_gx, st);
  int *dpiv = static_cast<int *>(ctx().buffer(kBufPiv, sizeof(int) * (size_t)n));
  ATLG_CHECK(cudaMemcpyAsync(dpiv, ipiv, sizeof(int) * n, cudaMemcpyHostToDevice, st));
  const int l_ga = l_lu, l_gb = l_lu;
  double *dgA = static_cast<double *>(ctx().buffer(kBufC, sizeof(double) * (size_t)l_ga * n));
  double *dgB = static_cast<double *>(ctx().buffer(kBufW6, sizeof(double) * (size_t)l_gb * (nrhs > 0 ? nrhs : 1)));
  if (nrhs > 0) {
    adjoint_dev(n, nrhs, dLU, l_lu, dpiv, dX, l_x, dgX, l_gx, dgA, l_ga, dgB, l_gb, st);
    to_host<double>(gB, ldgb, dgB, l_gb, n, nrhs, st);
  } else {
    dev_gescal(n, n, 0.0, dgA, l_ga, st);
  }
  to_host<double>(gA, ldga, dgA, l_ga, n, n, st);
  ATLG_CHECK(cudaStreamSynchronize(st));
  check_status(rout);
  return 0;
}

// ============================================================ C ABI: device
int atlg_num_sms(void) { return ctx().num_sms; }

void *atlg_stream(void) { return ctx().stream; }

unsigned atlg_status(void) {
  return gemm_status_read_and_clear() | lu_status_read_and_clear() | split_status_read_and_clear() |
         tf32_status_read_and_clear() | trsv_status_read_and_clear();
}

int atlg_sgemm_tf32x3_dev(int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb,
                          float *C, int ldc, void *stream) {
  if (M < 0 || N < 0 || K < 0) return -1;
  if (M == 0 || N == 0 || K == 0) return 0;
  cudaStream_t st = stream_of(stream);
  float *Ap = static_cast<float *>(ctx().buffer(kBufT0, sizeof(float) * tf32x3_packed_floats(M, K, false)));
  float *Bp = static_cast<float *>(ctx().buffer(kBufT1, sizeof(float) * tf32x3_packed_floats(N, K, true)));
  dev_sgemm_tf32x3_pack_a(M, K, A, lda, Ap, st);
  dev_sgemm_tf32x3_pack_b(K, N, B, ldb, Bp, st);
  dev_sgemm_tf32x3_packed(M, N, K, alpha, Ap, Bp, N, 0, C, ldc, st);
  return 0;
}

int atlg_dgemm_split_dev(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda,
                         const double *B, int ldb, double beta, double *C, int ldc, int nslices, void *stream) {
  if (M < 0 || N < 0 || K < 0 || nslices < 1 || nslices > 8) return -1;
  dev_dgemm_split(TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, nslices, stream_of(stream));
  return 0;
}

unsigned long long atlg_launch_count(void) { return ctx().launches; }

void atlg_prof_enable(int on) { ctx().prof = on != 0; }

// Sum of the recorded GEMM launches since the last collect: total device
// milliseconds, algorithmic flops and launch count.  Synchronizes.
int atlg_prof_collect(double *ms, double *flops, int *count) {
  Context &c = ctx();
  double t = 0.0, f = 0.0;
  int n = 0;
  for (auto &r : c.recs) {
    ATLG_CHECK(cudaEventSynchronize(r.end));
    float x = 0.f;
    ATLG_CHECK(cudaEventElapsedTime(&x, r.beg, r.end));
    t += x;
    f += r.flops;
    ++n;
    c.pool.push_back(r.beg);
    c.pool.push_back(r.end);
  }
  c.recs.clear();
  if (ms) *ms = t;
  if (flops) *flops = f;
  if (count) *count = n;
  return 0;
}

void atlg_prof_panels(int on) { ctx().prof_panels = on != 0; }

// LU panel launches recorded since the last collect, in stream order: the
// summed panel time (event before to event after each launch on the
// factorization's stream) and the summed gaps between one panel's end and the
// next panel's start (the step's remaining work on that stream, including
// waits for the side stream).  Synchronizes.
int atlg_prof_panels_collect(double *panel_ms, double *gap_ms, int *count) {
  Context &c = ctx();
  double p = 0.0, g = 0.0;
  int n = 0;
  for (size_t i = 0; i < c.panel_recs.size(); ++i) {
    auto &r = c.panel_recs[i];
    ATLG_CHECK(cudaEventSynchronize(r.end));
    float x = 0.f;
    ATLG_CHECK(cudaEventElapsedTime(&x, r.beg, r.end));
    p += x;
    if (i + 1 < c.panel_recs.size()) {
      ATLG_CHECK(cudaEventSynchronize(c.panel_recs[i + 1].beg));
      ATLG_CHECK(cudaEventElapsedTime(&x, r.end, c.panel_recs[i + 1].beg));
      g += x;
    }
    ++n;
  }
  for (auto &r : c.panel_recs) {
    c.pool.push_back(r.beg);
    c.pool.push_back(r.end);
  }
  c.panel_recs.clear();
  if (panel_ms) *panel_ms = p;
  if (gap_ms) *gap_ms = g;
  if (count) *count = n;
  return 0;
}

void atlg_probe_fp64_mma(double *m8n8k4, double *m16n8k4, double *m16n8k16) {
  probe_fp64_mma_tflops(m8n8k4, m16n8k4, m16n8k16);
}
void atlg_probe_peaks(double *fp64_tflops, double *fp32_tflops) {
  if (fp64_tflops) *fp64_tflops = probe_fp64_tflops();
  if (fp32_tflops) *fp32_tflops = probe_fp32_tflops();
}

int atlg_dgemm_dev(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
                   int ldb, double beta, double *C, int ldc, void *stream) {
  if (M < 0 || N < 0 || K < 0) return -1;
  dev_dgemm(TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, stream_of(stream));
  return 0;
}
int atlg_dgemm_dev_opts(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda,
                        const double *B, int ldb, double beta, double *C, int ldc, int allow_tma, void *stream) {
  if (M < 0 || N < 0 || K < 0) return -1;
  GemmOpts o;
  o.allow_tma = allow_tma != 0;
  dev_dgemm(TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, stream_of(stream), o);
  return 0;
}
int atlg_sgemm_dev(int TA, int TB, int M, int N, int K, float alpha, const float *A, int lda, const float *B,
                   int ldb, float beta, float *C, int ldc, void *stream) {
  if (M < 0 || N < 0 || K < 0) return -1;
  dev_sgemm(TA, TB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, stream_of(stream));
  return 0;
}
int atlg_dtrsm_dev(int Side, int Uplo, int TA, int Diag, int M, int N, double alpha, const double *A, int lda,
                   double *B, int ldb, void *stream) {
  if (M < 0 || N < 0) return -1;
  dev_dtrsm(Side, Uplo, TA, Diag, M, N, alpha, A, lda, B, ldb, stream_of(stream));
  return 0;
}
int atlg_dlaswp_dev(int N, double *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows, void *stream) {
  dev_dlaswp(N, A, lda, K1, K2, ipiv, inci, nrows, stream_of(stream));
  return 0;
}
int atlg_idamax_dev(int N, const double *X, int incX, int *result, void *stream) {
  return iamax_dev<double>(N, X, incX, result, stream);
}
int atlg_isamax_dev(int N, const float *X, int incX, int *result, void *stream) {
  return iamax_dev<float>(N, X, incX, result, stream);
}
void atlg_panel_cluster(int on) { set_panel_cluster(on != 0); }
void atlg_panel_split(int on) { set_panel_split(on != 0); }
void atlg_lu_defer_rows(int rows) { set_defer_rows(rows); }
void atlg_panel_fuse(int on) { set_panel_fuse(on != 0); }
void atlg_refine_trsv(int chained) { set_refine_trsv_chained(chained != 0); }
void atlg_panel_grid(int ctas) { set_panel_grid(ctas); }
void atlg_split_lu_leaf(int nb) { set_split_lu_leaf(nb); }
void atlg_panel_width(int w) { set_panel_width_f64(w); }
int atlg_dgetrf_dev(int M, int N, double *A, int lda, int *ipiv, int *info, void *stream) {
  if (M < 0 || N < 0 || lda < (M > 1 ? M : 1)) return -1;
  dev_dgetrf(M, N, A, lda, ipiv, info, stream_of(stream));
  return 0;
}
int atlg_sgetrf_dev(int M, int N, float *A, int lda, int *ipiv, int *info, void *stream) {
  if (M < 0 || N < 0 || lda < (M > 1 ? M : 1)) return -1;
  dev_sgetrf(M, N, A, lda, ipiv, info, stream_of(stream));
  return 0;
}
int atlg_sgetrf_tc_dev(int M, int N, float *A, int lda, int *ipiv, int *info, void *stream) {
  if (M < 0 || N < 0 || lda < (M > 1 ? M : 1)) return -1;
  dev_sgetrf_tc(M, N, A, lda, ipiv, info, stream_of(stream));
  return 0;
}
int atlg_dlag2s_dev(int M, int N, const double *A, int lda, float *SA, int ldsa, void *stream) {
  if (M < 0 || N < 0 || lda < (M > 1 ? M : 1) || ldsa < (M > 1 ? M : 1)) return -1;
  return dev_dlag2s(M, N, A, lda, SA, ldsa, stream_of(stream));
}
int atlg_dgesv_mixed_dev(int N, int NRHS, double *A, int lda, int *ipiv, const double *B, int ldb, double *X,
                         int ldx, double *berr, double *ferr, int *iters, int *status, void *stream) {
  if (N < 0 || NRHS < 0) return -1;
  return mixed_dev(N, NRHS, A, lda, ipiv, B, ldb, X, ldx, berr, ferr, iters, status, stream_of(stream));
}
int atlg_dgesv_adjoint_dev(int n, int nrhs, const double *LU, int lda, const int *ipiv, const double *X, int ldx,
                           const double *gX, int ldgx, double *gA, int ldga, double *gB, int ldgb, void *stream) {
  if (n < 0 || nrhs < 0) return -1;
  adjoint_dev(n, nrhs, LU, lda, ipiv, X, ldx, gX, ldgx, gA, ldga, gB, ldgb, stream_of(stream));
  return 0;
}
int atlg_dsyrk_dev(int Uplo, int Trans, int N, int K, double alpha, const double *A, int lda, double beta,
                   double *C, int ldc, void *stream) {
  if (N < 0 || K < 0) return -1;
  dev_dsyrk(Uplo, Trans == kNoTrans ? kNoTrans : kTrans, N, K, alpha, A, lda, beta, C, ldc, stream_of(stream));
  return 0;
}
int atlg_dpotrf_dev(int Uplo, int N, double *A, int lda, void *stream) {
  if (N < 0 || lda < (N > 1 ? N : 1)) return -1;
  return dev_dpotrf(Uplo, N, A, lda, stream_of(stream));
}
int atlg_dpotrs_dev(int Order, int Uplo, int N, int NRHS, const double *A, int lda, double *B, int ldb,
                    void *stream) {
  if (N < 0 || NRHS < 0) return -1;
  dev_dpotrs(Order, Uplo, N, NRHS, A, lda, B, ldb, stream_of(stream));
  return 0;
}
int atlg_dtrmm_dev(int Side, int Uplo, int TA, int Diag, int M, int N, double alpha, const double *A, int lda,
                   double *B, int ldb, void *stream) {
  if (M < 0 || N < 0) return -1;
  dev_dtrmm(Side, Uplo, TA, Diag, M, N, alpha, A, lda, B, ldb, stream_of(stream));
  return 0;
}
int atlg_dgemv_dev(int TA, int M, int N, double alpha, const double *A, int lda, const double *X, int incX,
                   double beta, double *Y, void *stream) {
  if (M < 0 || N < 0 || incX == 0) return -1;
  const int lx = (TA == kNoTrans) ? N : M, ly = (TA == kNoTrans) ? M : N;
  if (incX < 0) X += (size_t)(lx - 1) * (size_t)(-incX);
  dev_dgemv(TA, ly, lx, alpha, A, lda, X, incX, beta, Y, stream_of(stream));
  return 0;
}
int atlg_dtrsv_dev(int Uplo, int TA, int Diag, int N, const double *A, int lda, double *X, void *stream) {
  if (N < 0) return -1;
  dev_dtrsv(Uplo, TA, Diag, N, A, lda, X, stream_of(stream));
  return 0;
}
size_t atlg_strsv_chain_ws(int N) { return N > 0 ? sizeof(float) * strsv_chain_ws_floats(N) : 0; }
int atlg_strsv_chain_prepare_dev(int Uplo, int Diag, int N, const float *A, int lda, float *ws, void *stream) {
  if (N < 0 || lda < (N > 1 ? N : 1) || (Uplo != kUpper && Uplo != kLower) || (Diag != kUnit && Diag != kNonUnit))
    return -1;
  if (N > 0 && (reinterpret_cast<uintptr_t>(ws) & 15) != 0) return -1;
  dev_strsv_chain_prepare(Uplo, Diag, N, A, lda, ws, stream_of(stream));
  return 0;
}
int atlg_strsv_chain_dev(int Uplo, int N, const float *A, int lda, const float *ws, float *X, void *stream) {
  if (N < 0 || lda < (N > 1 ? N : 1) || (Uplo != kUpper && Uplo != kLower)) return -1;
  if (N > 0 && (reinterpret_cast<uintptr_t>(ws) & 15) != 0) return -1;
  dev_strsv_chain(Uplo, N, A, lda, ws, X, stream_of(stream));
  return 0;
}
int atlg_dtrtri_dev(int Order, int Uplo, int Diag, int N, double *A, int lda, void *stream) {
  if (N < 0 || lda < (N > 1 ? N : 1)) return -1;
  return dev_dtrtri(Order, Uplo, Diag, N, A, lda, stream_of(stream));
}
int atlg_dgetri_dev(int N, double *A, int lda, const int *ipiv, void *stream) {
  if (N < 0 || lda < (N > 1 ? N : 1)) return -1;
  if (N == 0) return 0;
  cudaStream_t st = stream_of(stream);
  std::vector<int> hp(N);
  ATLG_CHECK(cudaMemcpyAsync(hp.data(), ipiv, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  return dev_dgetri(N, A, lda, hp.data(), st);
}
int atlg_dgetrf_split_dev(int N, double *A, int lda, int *ipiv, int nslices, int nb, void *stream) {
  if (N < 0 || lda < (N > 1 ? N : 1) || nslices < 1 || nslices > 8 || nb < 256) return -1;
  return dev_dgetrf_split(N, A, lda, ipiv, nslices, nb, stream_of(stream));
}
int atlg_dgetrs_dev(int Order, int Trans, int N, int NRHS, const double *A, int lda, const int *ipiv, double *B,
                    int ldb, void *stream) {
  if (N < 0 || NRHS < 0) return -1;
  dev_dgetrs(Order, Trans, N, NRHS, A, lda, ipiv, B, ldb, stream_of(stream));
  return 0;
}

}  // extern "C"
