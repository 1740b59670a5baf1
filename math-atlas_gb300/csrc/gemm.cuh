// gemm.cuh -- device-pointer GEMM entry points used by the C ABI and by the
// LU / TRSM / refinement drivers.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

struct GemmOpts {
  bool allow_tma = true;   // false forces the cp.async loader (tests cover both)
  int num_sms = 0;         // 0: the device's SM count
  bool allow_gemv = true;  // N == 1 goes to the matrix-vector kernels
  int uplo = 0;            // kLower / kUpper: update only that triangle of C (M == N), as SYRK
  int tri = 0;             // triangular operand (TRMM): kTriA|kTriB, kTriUpper, kTriUnit; 0 = dense
  // batch of products of one shape: product z uses A + z*stride_a,
  // B + z*stride_b, C + z*stride_c (elements); batch > 1 uses the cp.async loader
  int batch = 1;
  long stride_a = 0, stride_b = 0, stride_c = 0;
};

// GemmOpts::tri bits.  The triangle is stated for op(A) (M x K, M == K) or
// op(B) (K x N, K == N); elements outside it are read as 0, the diagonal as 1
// when kTriUnit is set, and k-tiles wholly outside it are skipped.
enum { kTriA = 1, kTriB = 2, kTriWhich = 3, kTriUpper = 4, kTriUnit = 8 };

// Column-major C = alpha*op(A)*op(B) + beta*C, all pointers on the device.
void dev_dgemm(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda,
               const double *B, int ldb, double beta, double *C, int ldc, cudaStream_t st,
               const GemmOpts &o = GemmOpts());
void dev_sgemm(int TA, int TB, int M, int N, int K, float alpha, const float *A, int lda,
               const float *B, int ldb, float beta, float *C, int ldc, cudaStream_t st,
               const GemmOpts &o = GemmOpts());
// y = alpha*op(A)*x + beta*y with M = length of y and K = length of x (op(A)
// is M x K; A is M x K for NoTrans, K x M for Trans); y contiguous.
void dev_dgemv(int TA, int M, int K, double alpha, const double *A, int lda, const double *x, int incx, double beta,
               double *y, cudaStream_t st);
void dev_sgemv(int TA, int M, int K, float alpha, const float *A, int lda, const float *x, int incx, float beta,
               float *y, cudaStream_t st);
void dev_gescal(int M, int N, double beta, double *C, int ldc, cudaStream_t st);
void dev_gescal(int M, int N, float beta, float *C, int ldc, cudaStream_t st);
unsigned gemm_status_read_and_clear();

}  // namespace atlg
