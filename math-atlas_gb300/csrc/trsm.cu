// trsm.cu -- triangular solve with multiple right-hand sides, FP64 and FP32,
// column-major, all Side/Uplo/Trans/Diag cases:
//   Left:  op(A) * X = alpha * B        Right:  X * op(A) = alpha * B
//
// Replaces ATL_trsm (AtlasBase/Clint/trsm-micro.base:200-425: recursive split
// with GEMM updates, in-cache blocked solves ATL_iptrsm :550-760 and the
// diagonal micro-solves utrsmL_* :1384-1652 that keep the diagonal as
// reciprocals).
//
// GB300 design: blocked right-looking solve with TB=64.  Each diagonal
// block is solved by a warp per right-hand side (Left) or per row (Right):
// lanes own rows (or columns) of the block, the solved component is
// broadcast with a shuffle, and the diagonal is applied as a precomputed
// reciprocal as in the reference.  The off-diagonal update is one GEMM per
// block step on the library's DFMA/FFMA GEMM.
#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "trsm.cuh"

namespace atlg {

constexpr int TB = 64;          // diagonal block size
constexpr int WARPS = 8;        // right-hand sides (or rows) per CTA

// Load op(A)[r0:r0+n, r0:r0+n] into shared memory as T[i][k] (row-major,
// padded) with reciprocal diagonal.
template <typename T>
__device__ void load_tri(const T *A, int lda, int ta, int r0, int n, T (*tri)[TB + 1], T *rinv, bool unit) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, k = e / n;
    const T v = (ta == kNoTrans) ? A[(r0 + i) + (size_t)(r0 + k) * lda] : A[(r0 + k) + (size_t)(r0 + i) * lda];
    tri[i][k] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) rinv[i] = unit ? T(1) : T(1) / tri[i][i];
  __syncthreads();
}

// Left diagonal block: solve T * x = b for each column of B[r0:r0+n, :].
// lower -> forward substitution, else backward.  Lane l owns rows l, l+32.
template <typename T>
__global__ void __launch_bounds__(WARPS * 32)
    trsm_diag_left(const T *__restrict__ A, int lda, int ta, int lower, int unit, int r0, int n, int ncols,
                   T *__restrict__ B, int ldb) {
  __shared__ T tri[TB][TB + 1];
  __shared__ T rinv[TB];
  load_tri(A, lda, ta, r0, n, tri, rinv, unit != 0);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = blockIdx.x * WARPS + w;
  if (col >= ncols) return;
  T *b = B + r0 + (size_t)col * ldb;
  T x0 = lane < n ? b[lane] : T(0);
  T x1 = lane + 32 < n ? b[lane + 32] : T(0);
  if (lower) {
    for (int k = 0; k < n; ++k) {
      T bk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
      bk *= rinv[k];
      if (lane == (k & 31)) { if (k < 32) x0 = bk; else x1 = bk; }
      if (lane > k && lane < n) x0 -= tri[lane][k] * bk;
      if (lane + 32 > k && lane + 32 < n) x1 -= tri[lane + 32][k] * bk;
    }
  } else {
    for (int k = n - 1; k >= 0; --k) {
      T bk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
      bk *= rinv[k];
      if (lane == (k & 31)) { if (k < 32) x0 = bk; else x1 = bk; }
      if (lane < k) x0 -= tri[lane][k] * bk;
      if (lane + 32 < k) x1 -= tri[lane + 32][k] * bk;
    }
  }
  if (lane < n) b[lane] = x0;
  if (lane + 32 < n) b[lane + 32] = x1;
}

// Right diagonal block: solve x * T = b for each row of B[:, c0:c0+n].
// upper -> forward over columns, else backward.  Lane l owns columns l, l+32.
template <typename T>
__global__ void __launch_bounds__(WARPS * 32)
    trsm_diag_right(const T *__restrict__ A, int lda, int ta, int upper, int unit, int c0, int n, int nrows,
                    T *__restrict__ B, int ldb) {
  __shared__ T tri[TB][TB + 1];
  __shared__ T rinv[TB];
  load_tri(A, lda, ta, c0, n, tri, rinv, unit != 0);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = blockIdx.x * WARPS + w;
  if (row >= nrows) return;
  T *b = B + row + (size_t)c0 * ldb;
  T x0 = lane < n ? b[(size_t)lane * ldb] : T(0);
  T x1 = lane + 32 < n ? b[(size_t)(lane + 32) * ldb] : T(0);
  if (upper) {
    for (int j = 0; j < n; ++j) {
      T bj = __shfl_sync(0xffffffffu, j < 32 ? x0 : x1, j & 31);
      bj *= rinv[j];
      if (lane == (j & 31)) { if (j < 32) x0 = bj; else x1 = bj; }
      if (lane > j && lane < n) x0 -= bj * tri[j][lane];
      if (lane + 32 > j && lane + 32 < n) x1 -= bj * tri[j][lane + 32];
    }
  } else {
    for (int j = n - 1; j >= 0; --j) {
      T bj = __shfl_sync(0xffffffffu, j < 32 ? x0 : x1, j & 31);
      bj *= rinv[j];
      if (lane == (j & 31)) { if (j < 32) x0 = bj; else x1 = bj; }
      if (lane < j) x0 -= bj * tri[j][lane];
      if (lane + 32 < j) x1 -= bj * tri[j][lane + 32];
    }
  }
  if (lane < n) b[(size_t)lane * ldb] = x0;
  if (lane + 32 < n) b[(size_t)(lane + 32) * ldb] = x1;
}

template <typename T>
static void gemm_any(int ta, int tb, int M, int N, int K, T alpha, const T *A, int lda, const T *B, int ldb, T beta,
                     T *C, int ldc, cudaStream_t st);
template <>
void gemm_any<double>(int ta, int tb, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
                      int ldb, double beta, double *C, int ldc, cudaStream_t st) {
  dev_dgemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st);
}
template <>
void gemm_any<float>(int ta, int tb, int M, int N, int K, float alpha, const float *A, int lda, const float *B,
                     int ldb, float beta, float *C, int ldc, cudaStream_t st) {
  dev_sgemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st);
}

// address of the op(A) block at op-row r, op-col c
template <typename T>
static const T *opblk(const T *A, int lda, int ta, int r, int c) {
  return ta == kNoTrans ? A + r + (size_t)c * lda : A + c + (size_t)r * lda;
}

template <typename T>
static void trsm_impl(int side, int uplo, int tA, int diag, int M, int N, T alpha, const T *A, int lda, T *B,
                      int ldb, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  if (alpha == T(0)) { dev_gescal(M, N, T(0), B, ldb, st); return; }
  if (alpha != T(1)) dev_gescal(M, N, alpha, B, ldb, st);
  const int ta = (tA == kNoTrans) ? kNoTrans : kTrans;
  const int unit = (diag == kUnit);
  const dim3 blk(WARPS * 32);
  if (side == kLeft) {
    const bool lower = (uplo == kLower) != (ta != kNoTrans);
    const int nb = (M + TB - 1) / TB;
    const dim3 grid((N + WARPS - 1) / WARPS);
    for (int s = 0; s < nb; ++s) {
      const int b = lower ? s : nb - 1 - s;
      const int r0 = b * TB, n = (M - r0 < TB) ? M - r0 : TB;
      trsm_diag_left<T><<<grid, blk, 0, st>>>(A, lda, ta, lower, unit, r0, n, N, B, ldb);
      note_launch();
      ATLG_CHECK(cudaGetLastError());
      if (lower && r0 + n < M)
        gemm_any<T>(ta, kNoTrans, M - r0 - n, N, n, T(-1), opblk(A, lda, ta, r0 + n, r0), lda, B + r0, ldb, T(1),
                    B + r0 + n, ldb, st);
      if (!lower && r0 > 0)
        gemm_any<T>(ta, kNoTrans, r0, N, n, T(-1), opblk(A, lda, ta, 0, r0), lda, B + r0, ldb, T(1), B, ldb, st);
    }
  } else {
    const bool upper = (uplo == kUpper) != (ta != kNoTrans);
    const int nb = (N + TB - 1) / TB;
    const dim3 grid((M + WARPS - 1) / WARPS);
    for (int s = 0; s < nb; ++s) {
      const int b = upper ? s : nb - 1 - s;
      const int c0 = b * TB, n = (N - c0 < TB) ? N - c0 : TB;
      trsm_diag_right<T><<<grid, blk, 0, st>>>(A, lda, ta, upper, unit, c0, n, M, B, ldb);
      note_launch();
      ATLG_CHECK(cudaGetLastError());
      if (upper && c0 + n < N)
        gemm_any<T>(kNoTrans, ta, M, N - c0 - n, n, T(-1), B + (size_t)c0 * ldb, ldb, opblk(A, lda, ta, c0, c0 + n),
                    lda, T(1), B + (size_t)(c0 + n) * ldb, ldb, st);
      if (!upper && c0 > 0)
        gemm_any<T>(kNoTrans, ta, M, c0, n, T(-1), B + (size_t)c0 * ldb, ldb, opblk(A, lda, ta, c0, 0), lda, T(1), B,
                    ldb, st);
    }
  }
}

void dev_dtrsm(int side, int uplo, int ta, int diag, int M, int N, double alpha, const double *A, int lda,
               double *B, int ldb, cudaStream_t st) {
  trsm_impl<double>(side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb, st);
}
void dev_strsm(int side, int uplo, int ta, int diag, int M, int N, float alpha, const float *A, int lda, float *B,
               int ldb, cudaStream_t st) {
  trsm_impl<float>(side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb, st);
}

// Unit-lower solve of the LU's top block, L11 * X = A12, for the right-hand
// sides A12 = A[k:k+n, c0:c0+ncols] (the left block solve without the
// generic driver's scaling).
void dev_trsm_llnu_block(const double *A, int lda, int k, int n, double *B, int ldb, int ncols, cudaStream_t st) {
  if (n <= 0 || ncols <= 0) return;
  const dim3 grid((ncols + WARPS - 1) / WARPS);
  trsm_diag_left<double><<<grid, WARPS * 32, 0, st>>>(A + k + (size_t)k * lda, lda, kNoTrans, 1, 1, 0, n, ncols,
                                                       B, ldb);
      note_launch();
  ATLG_CHECK(cudaGetLastError());
}
void dev_trsm_llnu_block(const float *A, int lda, int k, int n, float *B, int ldb, int ncols, cudaStream_t st) {
  if (n <= 0 || ncols <= 0) return;
  const dim3 grid((ncols + WARPS - 1) / WARPS);
  trsm_diag_left<float><<<grid, WARPS * 32, 0, st>>>(A + k + (size_t)k * lda, lda, kNoTrans, 1, 1, 0, n, ncols, B,
                                                      ldb);
      note_launch();
  ATLG_CHECK(cudaGetLastError());
}

}  // namespace atlg
