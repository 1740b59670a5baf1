// chol.cu -- SYRK and the Cholesky path: cblas_?syrk, clapack_?potrf,
// clapack_?potrs, clapack_?posv on GB300, FP64 and FP32.
//
// Reference path replaced: the SYRK interface (AtlasBase/Clint/cblas.base:
// 339-450), ATL_potrf (AtlasBase/Clint/atlas-lp.base:332-374) with the
// recursive ATL_potrfU / ATL_potrfL (:675-968: split in halves, factor the
// left half, TRSM the off-diagonal block, SYRK the trailing block, recurse)
// and ATL_potrs (:969-1052).
//
// GB300 design: right-looking blocked Cholesky, block 64.  The 64 x 64
// diagonal block is factored by one CTA in shared memory (column by column:
// square root of the pivot, reciprocal scaling, rank-1 update); the block
// below (Lower) or to the right (Upper) is a TRSM on the blocked solver of
// trsm.cu; the trailing update is the DFMA/FFMA GEMM restricted to one
// triangle (tiles wholly outside the triangle exit at once).  Like the
// reference, the factorization stops at the first non-positive pivot and
// returns its 1-based index, leaving that pivot's value in place.
#include <math.h>

#include "chol.cuh"
#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "trsm.cuh"

namespace atlg {

constexpr int CB = 64;

// Scale the `uplo` triangle of the n x n matrix C by beta (beta == 0 stores zeros).
template <typename T>
__global__ void tri_scale_kernel(int n, int uplo, T beta, T *C, int ldc) {
  const long total = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    if ((uplo == kLower && i < j) || (uplo == kUpper && i > j)) continue;
    T *c = C + i + (size_t)j * ldc;
    *c = (beta == T(0)) ? T(0) : beta * *c;
  }
}

template <typename T>
static void gemm_tri(int ta, int tb, int n, int k, T alpha, const T *A, int lda, T beta, T *C, int ldc, int uplo,
                     cudaStream_t st) {
  GemmOpts o;
  o.uplo = uplo;
  if (sizeof(T) == 8)
    dev_dgemm(ta, tb, n, n, k, (double)alpha, (const double *)A, lda, (const double *)A, lda, (double)beta,
              (double *)C, ldc, st, o);
  else
    dev_sgemm(ta, tb, n, n, k, (float)alpha, (const float *)A, lda, (const float *)A, lda, (float)beta,
              (float *)C, ldc, st, o);
}

// C = alpha * op(A) op(A)^T + beta * C on the `uplo` triangle, column-major.
// trans == NoTrans: A is n x k, C = A A^T;  otherwise A is k x n, C = A^T A.
template <typename T>
static void syrk_impl(int uplo, int trans, int n, int k, T alpha, const T *A, int lda, T beta, T *C, int ldc,
                      cudaStream_t st) {
  if (n <= 0) return;
  if (alpha == T(0) || k <= 0) {
    if (beta != T(1)) {
      const long total = (long)n * n;
      int blocks = (int)((total + 255) / 256);
      if (blocks > 4096) blocks = 4096;
      tri_scale_kernel<T><<<blocks, 256, 0, st>>>(n, uplo, beta, C, ldc);
      note_launch();
      ATLG_CHECK(cudaGetLastError());
    }
    return;
  }
  if (trans == kNoTrans) gemm_tri<T>(kNoTrans, kTrans, n, k, alpha, A, lda, beta, C, ldc, uplo, st);
  else gemm_tri<T>(kTrans, kNoTrans, n, k, alpha, A, lda, beta, C, ldc, uplo, st);
}

void dev_dsyrk(int uplo, int trans, int n, int k, double alpha, const double *A, int lda, double beta, double *C,
               int ldc, cudaStream_t st) {
  syrk_impl<double>(uplo, trans, n, k, alpha, A, lda, beta, C, ldc, st);
}
void dev_ssyrk(int uplo, int trans, int n, int k, float alpha, const float *A, int lda, float beta, float *C,
               int ldc, cudaStream_t st) {
  syrk_impl<float>(uplo, trans, n, k, alpha, A, lda, beta, C, ldc, st);
}

// Copy the strict upper triangle of the n x n matrix C to the lower one
// (ATL_syreflect, used by cblas_dgemm's A A^T shortcut).  32 x 32 tiles
// through shared memory so both the read and the write are coalesced.
template <typename T>
__global__ void syreflect_kernel(int n, T *C, int ldc) {
  __shared__ T t[32][33];
  const int bi = blockIdx.y * 32, bj = blockIdx.x * 32;   // destination tile rows bi.., cols bj..
  if (bj > bi) return;                                     // tiles wholly above the diagonal
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < 32; r += 8) {                       // source: rows bj.., cols bi.. (upper part)
    const int i = bj + tx, j = bi + r;
    if (i < n && j < n) t[r][tx] = C[i + (size_t)j * ldc];
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = bi + tx, j = bj + r;
    if (i < n && j < n && i > j) C[i + (size_t)j * ldc] = t[tx][r];
  }
}

template <typename T>
static void syreflect_impl(int n, T *C, int ldc, cudaStream_t st) {
  if (n <= 1) return;
  const int nt = (n + 31) / 32;
  syreflect_kernel<T><<<dim3(nt, nt), dim3(32, 8), 0, st>>>(n, C, ldc);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}
void dev_dsyreflect(int n, double *C, int ldc, cudaStream_t st) { syreflect_impl<double>(n, C, ldc, st); }
void dev_ssyreflect(int n, float *C, int ldc, cudaStream_t st) { syreflect_impl<float>(n, C, ldc, st); }

// Factor the nb x nb diagonal block at A (nb <= 64) in shared memory, as
// L L^T (Lower) or U^T U (Upper, handled as the transpose).  One barrier per
// column: step j applies the rank-1 update with the scaled column computed on
// the fly (column j itself is scaled in step j+1, when nothing reads it any
// more).  The square root and reciprocal of each pivot are computed once, by
// the thread that finishes that diagonal entry, and read from shared memory
// (FP64 division and square root are expensive on GB300's FP64 pipe).  Four
// threads share a row.  On a non-positive pivot j the block keeps that value,
// *info gets koff + j + 1 and the factorization stops.
template <typename T>
__global__ void __launch_bounds__(256) potf2_kernel(int nb, int uplo, T *A, int lda, int koff, int *info) {
  __shared__ T a[CB][CB + 1];
  __shared__ T s_sq[3], s_rc[3];   // by step mod 3: step j reads j and j-1, writes j+1
  __shared__ int s_ok[3];
  const int tid = threadIdx.x;
  const int row = tid >> 2, q = tid & 3;
  for (int e = tid; e < nb * nb; e += 256) {
    const int i = e % nb, k = e / nb;
    if (i >= k) a[i][k] = (uplo == kLower) ? A[i + (size_t)k * lda] : A[k + (size_t)i * lda];
  }
  __syncthreads();
  auto pivot = [&](int j) {   // one thread: pivot j's square root and reciprocal
    const T ajj = a[j][j];
    const int ok = ajj > T(0);
    const T sj = ok ? sqrt(ajj) : T(0);
    s_sq[j % 3] = sj;
    s_rc[j % 3] = ok ? T(1) / sj : T(0);
    s_ok[j % 3] = ok;
  };
  if (tid == 0) pivot(0);
  __syncthreads();
  int fail = 0;
  for (int j = 0; j < nb; ++j) {
    const int b = j % 3, bp = (j + 2) % 3;
    if (j > 0 && q == 0) {   // finish column j-1
      if (row == j - 1) a[row][row] = s_sq[bp];
      else if (row > j - 1 && row < nb) a[row][j - 1] *= s_rc[bp];
    }
    if (!s_ok[b]) { fail = j + 1; break; }   // same in every thread
    const T r = s_rc[b];
    if (row > j && row < nb) {
      const T lij = a[row][j] * r;
      for (int k = j + 1 + q; k <= row; k += 4) a[row][k] -= lij * (a[k][j] * r);
      // the thread that just finished a[j+1][j+1] prepares the next pivot
      if (row == j + 1 && q == 0) pivot(j + 1);
    }
    __syncthreads();
  }
  if (!fail && q == 0 && row == nb - 1) a[row][row] = s_sq[(nb - 1) % 3];
  __syncthreads();
  // write back the processed columns (the failing pivot column as it stands)
  const int done = fail ? fail : nb;
  for (int e = tid; e < nb * nb; e += 256) {
    const int i = e % nb, k = e / nb;
    if (i < k || k >= done) continue;
    if (uplo == kLower) A[i + (size_t)k * lda] = a[i][k];
    else A[k + (size_t)i * lda] = a[i][k];
  }
  if (tid == 0 && fail && *info == 0) *info = koff + fail;
}

template <typename T>
static void trsm_any(int side, int uplo, int ta, int diag, int M, int N, const T *A, int lda, T *B, int ldb,
                     cudaStream_t st) {
  if (sizeof(T) == 8)
    dev_dtrsm(side, uplo, ta, diag, M, N, 1.0, (const double *)A, lda, (double *)B, ldb, st);
  else
    dev_strsm(side, uplo, ta, diag, M, N, 1.0f, (const float *)A, lda, (float *)B, ldb, st);
}

// Column-major Cholesky of the `uplo` triangle.  Returns the reference's
// info: 0, or the 1-based index of the first non-positive pivot.
template <typename T>
static int potrf_impl(int uplo, int n, T *A, int lda, cudaStream_t st) {
  if (n <= 0) return 0;
  Context &c = ctx();
  int *dinfo = static_cast<int *>(c.buffer(kBufChol, 64));
  ATLG_CHECK(cudaMemsetAsync(dinfo, 0, sizeof(int), st));
  int hinfo = 0;
  for (int k = 0; k < n; k += CB) {
    const int jb = (n - k < CB) ? n - k : CB;
    T *Akk = A + k + (size_t)k * lda;
    potf2_kernel<T><<<1, 256, 0, st>>>(jb, uplo, Akk, lda, k, dinfo);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    // the reference stops at the first failing pivot: look before updating
    ATLG_CHECK(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
    ATLG_CHECK(cudaStreamSynchronize(st));
    if (hinfo) return hinfo;
    const int m = n - k - jb;
    if (m <= 0) break;
    if (uplo == kLower) {
      T *A21 = A + (k + jb) + (size_t)k * lda;
      trsm_any<T>(kRight, kLower, kTrans, kNonUnit, m, jb, Akk, lda, A21, lda, st);
      gemm_tri<T>(kNoTrans, kTrans, m, jb, T(-1), A21, lda, T(1), A + (k + jb) + (size_t)(k + jb) * lda, lda,
                  kLower, st);
    } else {
      T *A12 = A + k + (size_t)(k + jb) * lda;
      trsm_any<T>(kLeft, kUpper, kTrans, kNonUnit, jb, m, Akk, lda, A12, lda, st);
      gemm_tri<T>(kTrans, kNoTrans, m, jb, T(-1), A12, lda, T(1), A + (k + jb) + (size_t)(k + jb) * lda, lda,
                  kUpper, st);
    }
  }
  return 0;
}

int dev_dpotrf(int uplo, int n, double *A, int lda, cudaStream_t st) { return potrf_impl<double>(uplo, n, A, lda, st); }
int dev_spotrf(int uplo, int n, float *A, int lda, cudaStream_t st) { return potrf_impl<float>(uplo, n, A, lda, st); }

// ATL_potrs (AtlasBase/Clint/atlas-lp.base:969-1052), cblas order handling
// of the two TRSMs as cblas_trsm does (RowMajor flips Side and Uplo).
template <typename T>
static void trsm_order(int order, int side, int uplo, int ta, int M, int N, const T *A, int lda, T *B, int ldb,
                       cudaStream_t st) {
  if (order == kRowMajor) {
    side = side == kLeft ? kRight : kLeft;
    uplo = uplo == kUpper ? kLower : kUpper;
    const int t = M; M = N; N = t;
  }
  trsm_any<T>(side, uplo, ta, kNonUnit, M, N, A, lda, B, ldb, st);
}

template <typename T>
static void potrs_impl(int order, int uplo, int n, int nrhs, const T *A, int lda, T *B, int ldb, cudaStream_t st) {
  if (!n || !nrhs) return;
  if (order == kColMajor) {
    if (uplo == kUpper) {
      trsm_order<T>(order, kLeft, kUpper, kTrans, n, nrhs, A, lda, B, ldb, st);
      trsm_order<T>(order, kLeft, kUpper, kNoTrans, n, nrhs, A, lda, B, ldb, st);
    } else {
      trsm_order<T>(order, kLeft, kLower, kNoTrans, n, nrhs, A, lda, B, ldb, st);
      trsm_order<T>(order, kLeft, kLower, kTrans, n, nrhs, A, lda, B, ldb, st);
    }
  } else {
    if (uplo == kUpper) {
      trsm_order<T>(order, kRight, kUpper, kNoTrans, nrhs, n, A, lda, B, ldb, st);
      trsm_order<T>(order, kRight, kUpper, kTrans, nrhs, n, A, lda, B, ldb, st);
    } else {
      trsm_order<T>(order, kRight, kLower, kTrans, nrhs, n, A, lda, B, ldb, st);
      trsm_order<T>(order, kRight, kLower, kNoTrans, nrhs, n, A, lda, B, ldb, st);
    }
  }
}

void dev_dpotrs(int order, int uplo, int n, int nrhs, const double *A, int lda, double *B, int ldb, cudaStream_t st) {
  potrs_impl<double>(order, uplo, n, nrhs, A, lda, B, ldb, st);
}
void dev_spotrs(int order, int uplo, int n, int nrhs, const float *A, int lda, float *B, int ldb, cudaStream_t st) {
  potrs_impl<float>(order, uplo, n, nrhs, A, lda, B, ldb, st);
}

}  // namespace atlg
