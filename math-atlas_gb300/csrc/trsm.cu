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
#include <mutex>

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
  // a warp per right-hand side; the CTA's triangle serves every column it visits
  for (int col = blockIdx.x * WARPS + w; col < ncols; col += gridDim.x * WARPS) {
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
  // a warp per row of B; the CTA's triangle serves every row it visits
  for (int row = blockIdx.x * WARPS + w; row < nrows; row += gridDim.x * WARPS) {
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

// CTAs of a diagonal-block solve over `count` columns (or rows): enough for
// four CTAs per SM, each reusing its triangle over the rest.
static int diag_grid(int count) {
  const int need = (count + WARPS - 1) / WARPS, cap = 4 * ctx().num_sms;
  return need < cap ? need : cap;
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
    const dim3 grid(diag_grid(N));
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
    const dim3 grid(diag_grid(M));
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

// ---------------------------------------------- left solves with block inverses
// For many right-hand sides (getrs with NRHS >= 8, the adjoint's transposed
// solves) the 64-step substitution of each diagonal block (one warp per
// right-hand side, a dependent chain) dominates its step.  Here every
// diagonal block of the stored triangle is inverted once (one CTA per block,
// column by column: X(0:j, j) = -inv(T(0:j,0:j)) T(0:j, j) / T(j,j)) into a
// workspace of 64 x 64 column-major blocks, and each step applies
// op(inv(T_bb)) to its rows of B as a small dense product; the updates of the
// other rows are the same GEMMs as trsm_impl's.  inv(op(T)) = op(inv(T)), so
// one set of inverses serves both op(A) = A and A^T.  Rounding differs from
// substitution.
template <typename T>
__global__ void __launch_bounds__(TB) trsm_inv_diag_kernel(int M, const T *__restrict__ A, int lda, int upper,
                                                           int unit, T *__restrict__ W) {
  __shared__ T a[TB][TB + 1];
  const int o = blockIdx.x * TB;
  const int nb = (M - o < TB) ? M - o : TB;
  const int tid = threadIdx.x;
  const T *Ab = A + o + (size_t)o * lda;
  // a = the block as an upper triangle (a lower block is inverted through its transpose)
  for (int e = tid; e < TB * TB; e += TB) {
    const int i = e % TB, k = e / TB;
    T v = T(0);
    if (i < nb && k < nb && i <= k) v = upper ? Ab[i + (size_t)k * lda] : Ab[k + (size_t)i * lda];
    a[i][k] = v;
  }
  __syncthreads();
  if (unit && tid < nb) a[tid][tid] = T(1);
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const T dinv = unit ? T(1) : T(1) / a[j][j];
    T t = T(0);
    if (tid < j)
      for (int k = tid; k < j; ++k) t = fma(a[tid][k], a[k][j], t);
    __syncthreads();
    if (tid < j) a[tid][j] = -dinv * t;
    if (tid == j) a[j][j] = dinv;
    __syncthreads();
  }
  T *Wb = W + (size_t)blockIdx.x * TB * TB;
  for (int e = tid; e < TB * TB; e += TB) {
    const int i = e % TB, k = e / TB;
    T v = T(0);
    if (i < nb && k < nb) v = upper ? (i <= k ? a[i][k] : T(0)) : (k <= i ? a[k][i] : T(0));
    Wb[e] = v;                                   // W(i, k), column-major
  }
}

// B(0:n, c) <- op(Wb) B(0:n, c) for 4 right-hand sides per CTA.
template <typename T>
__global__ void __launch_bounds__(256) trsm_inv_apply_kernel(const T *__restrict__ Wb, int ta, int n, int N, T *B,
                                                             int ldb) {
  __shared__ T w[TB][TB + 1];
  __shared__ T bs[4][TB];
  const int tid = threadIdx.x, i = tid & (TB - 1), cl = tid >> 6;
  const int c = blockIdx.x * 4 + cl;
  for (int e = tid; e < TB * TB; e += 256) w[e / TB][e % TB] = Wb[e];   // w[k][r] = W(r, k)
  bs[cl][i] = (c < N && i < n) ? B[i + (size_t)c * ldb] : T(0);
  __syncthreads();
  T acc = T(0);
  if (ta == kNoTrans) {
    for (int k = 0; k < n; ++k) acc = fma(w[k][i], bs[cl][k], acc);     // W(i, k)
  } else {
    for (int k = 0; k < n; ++k) acc = fma(w[i][k], bs[cl][k], acc);     // W(k, i)
  }
  if (c < N && i < n) B[i + (size_t)c * ldb] = acc;
}

template <typename T>
static void trsm_left_inv_impl(int uplo, int tA, int diag, int M, int N, const T *A, int lda, T *B, int ldb,
                               cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  const int ta = (tA == kNoTrans) ? kNoTrans : kTrans;
  const int unit = (diag == kUnit);
  const bool lower = (uplo == kLower) != (ta != kNoTrans);   // of op(A)
  const int nb = (M + TB - 1) / TB;
  T *W = static_cast<T *>(ctx().buffer(kBufTrsmInv, sizeof(T) * (size_t)nb * TB * TB));
  trsm_inv_diag_kernel<T><<<nb, TB, 0, st>>>(M, A, lda, uplo == kUpper ? 1 : 0, unit, W);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
  const int gridN = (N + 3) / 4;
  for (int s = 0; s < nb; ++s) {
    const int b = lower ? s : nb - 1 - s;
    const int r0 = b * TB, n = (M - r0 < TB) ? M - r0 : TB;
    trsm_inv_apply_kernel<T><<<gridN, 256, 0, st>>>(W + (size_t)b * TB * TB, ta, n, N, B + r0, ldb);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    if (lower && r0 + n < M)
      gemm_any<T>(ta, kNoTrans, M - r0 - n, N, n, T(-1), opblk(A, lda, ta, r0 + n, r0), lda, B + r0, ldb, T(1),
                  B + r0 + n, ldb, st);
    if (!lower && r0 > 0)
      gemm_any<T>(ta, kNoTrans, r0, N, n, T(-1), opblk(A, lda, ta, 0, r0), lda, B + r0, ldb, T(1), B, ldb, st);
  }
}

void dev_dtrsm_left_inv(int uplo, int ta, int diag, int M, int N, const double *A, int lda, double *B, int ldb,
                        cudaStream_t st) {
  trsm_left_inv_impl<double>(uplo, ta, diag, M, N, A, lda, B, ldb, st);
}
void dev_strsm_left_inv(int uplo, int ta, int diag, int M, int N, const float *A, int lda, float *B, int ldb,
                        cudaStream_t st) {
  trsm_left_inv_impl<float>(uplo, ta, diag, M, N, A, lda, B, ldb, st);
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
  const dim3 grid(diag_grid(ncols));
  trsm_diag_left<double><<<grid, WARPS * 32, 0, st>>>(A + k + (size_t)k * lda, lda, kNoTrans, 1, 1, 0, n, ncols,
                                                       B, ldb);
      note_launch();
  ATLG_CHECK(cudaGetLastError());
}
// FP32 form: a thread per right-hand side, its column in registers, the
// triangle's columns read as shared-memory broadcasts.  Each element gets
// the same fused multiply-adds in the same order as in trsm_diag_left
// (x_i -= L_ik x_k for k = 0, 1, ..., i-1; the unit diagonal's reciprocal
// is 1), so the result is bit-identical; the latency chain is one thread's
// FMAs instead of a shuffle per row, and the FP32 pipe is not the limit.
constexpr int kColsPerCta = 128;
constexpr size_t kColsSmem = sizeof(float) * ((size_t)TB * TB + (size_t)kColsPerCta * (TB + 1));

__global__ void __launch_bounds__(kColsPerCta)
    trsm_llnu_cols_kernel(const float *__restrict__ L, int lda, int n, int ncols, float *__restrict__ B, int ldb) {
  extern __shared__ float cs_smem[];
  float *tri = cs_smem;                      // column-major: tri[k * TB + i] = L(i, k), strictly lower, 0 elsewhere
  float *xs = cs_smem + TB * TB;             // column c of the strip at xs[c * (TB + 1) + i]
  const int t = threadIdx.x;
  const int c0 = blockIdx.x * kColsPerCta;
  for (int e = t; e < TB * TB; e += kColsPerCta) {
    const int i = e & (TB - 1), k = e / TB;
    tri[e] = (k < i && i < n) ? L[i + (size_t)k * lda] : 0.f;
  }
  for (int e = t; e < kColsPerCta * TB; e += kColsPerCta) {
    const int i = e & (TB - 1), c = e / TB;
    xs[c * (TB + 1) + i] = (i < n && c0 + c < ncols) ? B[i + (size_t)(c0 + c) * ldb] : 0.f;
  }
  __syncthreads();
  float x[TB];
#pragma unroll
  for (int i = 0; i < TB; ++i) x[i] = xs[t * (TB + 1) + i];
#pragma unroll
  for (int k = 0; k < TB - 1; ++k) {
    const float xk = x[k];
#pragma unroll
    for (int i = k + 1; i < TB; ++i) x[i] = fmaf(-tri[k * TB + i], xk, x[i]);
  }
#pragma unroll
  for (int i = 0; i < TB; ++i) xs[t * (TB + 1) + i] = x[i];
  __syncthreads();
  for (int e = t; e < kColsPerCta * TB; e += kColsPerCta) {
    const int i = e & (TB - 1), c = e / TB;
    if (i < n && c0 + c < ncols) B[i + (size_t)(c0 + c) * ldb] = xs[c * (TB + 1) + i];
  }
}

void dev_trsm_llnu_block(const float *A, int lda, int k, int n, float *B, int ldb, int ncols, cudaStream_t st) {
  if (n <= 0 || ncols <= 0) return;
  if (n <= TB) {
    static std::once_flag once;
    std::call_once(once, [] {
      ATLG_CHECK(cudaFuncSetAttribute(trsm_llnu_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kColsSmem));
    });
    trsm_llnu_cols_kernel<<<(ncols + kColsPerCta - 1) / kColsPerCta, kColsPerCta, kColsSmem, st>>>(
        A + k + (size_t)k * lda, lda, n, ncols, B, ldb);
  } else {
    const dim3 grid(diag_grid(ncols));
    trsm_diag_left<float><<<grid, WARPS * 32, 0, st>>>(A + k + (size_t)k * lda, lda, kNoTrans, 1, 1, 0, n, ncols,
                                                        B, ldb);
  }
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

}  // namespace atlg

// ---------------------------------------------------------------- TRSV
// One right-hand side (the solve after a factorization): a single launch
// with one CTA per 64-row block.  CTAs take blocks in solve order from an
// atomic ticket; a CTA folds in the contribution of every earlier block as
// soon as that block's flag is published, then solves its diagonal block
// (warp substitution, reciprocal diagonal) and publishes its piece of x.  A
// CTA only waits on blocks whose tickets were taken before its own, so every
// block it waits for is running or done; every wait is bounded.
namespace atlg {

__device__ unsigned g_trsv_status;
constexpr int TV_B = 64;
constexpr unsigned kFlagPollLimit = 1u << 24;

// INV: the CTA inverts its diagonal block while it waits for the earlier
// blocks (off the solve's critical path), and its block of x is then one
// 64 x 64 product by the inverse instead of a 64-step substitution.
template <typename T, bool INV>
__global__ void __launch_bounds__(256)
    trsv_lookback_kernel(int n, const T *__restrict__ A, int lda, int ta, int lower, int unit, T *x, int *flags,
                         int *ticket) {
  __shared__ T tri[TV_B][TV_B + 1];
  __shared__ T tinv[INV ? TV_B : 1][TV_B + 1];
  __shared__ T ys[TV_B];
  __shared__ T rinv[TV_B];
  __shared__ T part[8][TV_B];
  __shared__ int s_b, s_fail;
  const int nb = (n + TV_B - 1) / TV_B;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    const int t = atomicAdd(ticket, 1);
    s_b = lower ? t : nb - 1 - t;
    s_fail = 0;
  }
  __syncthreads();
  const int b = s_b;
  const int r0 = b * TV_B;
  const int nr = (n - r0 < TV_B) ? n - r0 : TV_B;
  // diagonal block of op(A), reciprocal diagonal
  for (int e = threadIdx.x; e < nr * nr; e += 256) {
    const int i = e % nr, k = e / nr;
    tri[i][k] = (ta == kNoTrans) ? A[(r0 + i) + (size_t)(r0 + k) * lda] : A[(r0 + k) + (size_t)(r0 + i) * lda];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += 256) rinv[i] = unit ? T(1) : T(1) / tri[i][i];
  if (INV) {
    __syncthreads();
    // column j of the inverse of the (op) diagonal block, one thread per column
    const int j = threadIdx.x;
    if (j < TV_B) {
      for (int i = 0; i < TV_B; ++i) tinv[i][j] = T(0);
      if (j < nr) {
        tinv[j][j] = rinv[j];
        if (lower) {
          for (int i = j + 1; i < nr; ++i) {
            T s = T(0);
            for (int k = j; k < i; ++k) s = fma(tri[i][k], tinv[k][j], s);
            tinv[i][j] = -s * rinv[i];
          }
        } else {
          for (int i = j - 1; i >= 0; --i) {
            T s = T(0);
            for (int k = i + 1; k <= j; ++k) s = fma(tri[i][k], tinv[k][j], s);
            tinv[i][j] = -s * rinv[i];
          }
        }
      }
    }
  }
  // contributions of earlier blocks: warp w takes columns k = c0 + w, w+8, ...
  T acc0 = T(0), acc1 = T(0);              // rows lane, lane+32 (op(A) = A)
  T accT[8];                               // rows w*8..w*8+7, lanes over k (op(A) = A^T)
#pragma unroll
  for (int q = 0; q < 8; ++q) accT[q] = T(0);
  for (int s = 0; s < nb - 1; ++s) {
    const int c = lower ? s : nb - 1 - s;
    if (lower ? c >= b : c <= b) break;
    const int c0 = c * TV_B;
    const int nc = (n - c0 < TV_B) ? n - c0 : TV_B;
    // this block's part of A does not depend on x: load it before waiting
    T pa[16];
    if (ta == kNoTrans) {
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const int k = w + 8 * m;
        const T *col = A + r0 + (size_t)(c0 + k) * lda;
        pa[2 * m] = (k < nc && lane < nr) ? col[lane] : T(0);
        pa[2 * m + 1] = (k < nc && lane + 32 < nr) ? col[lane + 32] : T(0);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = w * 8 + q;
        pa[2 * q] = (i < nr && lane < nc) ? A[(c0 + lane) + (size_t)(r0 + i) * lda] : T(0);
        pa[2 * q + 1] = (i < nr && lane + 32 < nc) ? A[(c0 + lane + 32) + (size_t)(r0 + i) * lda] : T(0);
      }
    }
    if (threadIdx.x == 0) {
      unsigned i = 0;
      while (atomicAdd(&flags[c], 0) == 0) {
        if (++i > kFlagPollLimit) { atomicOr(&g_trsv_status, kErrGridTimeout); s_fail = 1; break; }
        if (i > 32) __nanosleep(64);
      }
      __threadfence();
    }
    __syncthreads();
    if (s_fail) return;
    if (ta == kNoTrans) {
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const int k = w + 8 * m;
        const T xk = (k < nc) ? __ldcg(x + c0 + k) : T(0);      // published by another CTA: read at L2
        acc0 = fma(pa[2 * m], xk, acc0);
        acc1 = fma(pa[2 * m + 1], xk, acc1);
      }
    } else {
      const T x0 = (lane < nc) ? __ldcg(x + c0 + lane) : T(0);
      const T x1 = (lane + 32 < nc) ? __ldcg(x + c0 + lane + 32) : T(0);
#pragma unroll
      for (int q = 0; q < 8; ++q) accT[q] = fma(pa[2 * q + 1], x1, fma(pa[2 * q], x0, accT[q]));
    }
  }
  // gather the partial sums: part[w][row]
  if (ta == kNoTrans) {
    part[w][lane] = acc0;
    part[w][lane + 32] = acc1;
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      T v = accT[q];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) part[0][w * 8 + q] = v;
    }
  }
  __syncthreads();
  if (INV) {
    if (w == 0) {
      T y0 = T(0), y1 = T(0);
      if (ta == kNoTrans) {
        for (int q = 0; q < 8; ++q) { y0 += part[q][lane]; y1 += part[q][lane + 32]; }
      } else {
        y0 = part[0][lane];
        y1 = part[0][lane + 32];
      }
      ys[lane] = lane < nr ? x[r0 + lane] - y0 : T(0);
      ys[lane + 32] = lane + 32 < nr ? x[r0 + lane + 32] - y1 : T(0);
    }
    __syncthreads();
    // x_i = sum_k inv[i][k] ys[k]: four threads per row, 16 terms each
    const int i = threadIdx.x >> 2, q = threadIdx.x & 3;
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) s = fma(tinv[i][q * 16 + k], ys[q * 16 + k], s);
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (q == 0 && i < nr) x[r0 + i] = s;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicExch(&flags[b], 1);
    return;
  }
  if (w == 0) {
    T y0 = T(0), y1 = T(0);
    if (ta == kNoTrans) {
      for (int q = 0; q < 8; ++q) { y0 += part[q][lane]; y1 += part[q][lane + 32]; }
    } else {
      y0 = part[0][lane];
      y1 = part[0][lane + 32];
    }
    T x0 = lane < nr ? x[r0 + lane] - y0 : T(0);
    T x1 = lane + 32 < nr ? x[r0 + lane + 32] - y1 : T(0);
    if (lower) {
      for (int k = 0; k < nr; ++k) {
        T bk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
        bk *= rinv[k];
        if (lane == (k & 31)) { if (k < 32) x0 = bk; else x1 = bk; }
        if (lane > k && lane < nr) x0 -= tri[lane][k] * bk;
        if (lane + 32 > k && lane + 32 < nr) x1 -= tri[lane + 32][k] * bk;
      }
    } else {
      for (int k = nr - 1; k >= 0; --k) {
        T bk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
        bk *= rinv[k];
        if (lane == (k & 31)) { if (k < 32) x0 = bk; else x1 = bk; }
        if (lane < k) x0 -= tri[lane][k] * bk;
        if (lane + 32 < k) x1 -= tri[lane + 32][k] * bk;
      }
    }
    if (lane < nr) x[r0 + lane] = x0;
    if (lane + 32 < nr) x[r0 + lane + 32] = x1;
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicExch(&flags[b], 1);
  }
}

// The mixed solver's FP32 refinement solves (op(A) = A): as the INV form of
// trsv_lookback_kernel, but a block publishes its piece of x as 64-bit words
// (float value, call epoch) and a waiting CTA polls those words themselves,
// so each value arrives with its signal -- one L2 round trip per block on the
// solve's critical path instead of a flag and then the data.  Words from
// earlier calls carry older epochs and are never taken.
__global__ void __launch_bounds__(256)
    trsv_tagged_kernel(int n, const float *__restrict__ A, int lda, int lower, int unit, float *x,
                       unsigned long long *pub, unsigned epoch, int *ticket) {
  __shared__ float tri[TV_B][TV_B + 1];
  __shared__ float tinv[TV_B][TV_B + 1];
  __shared__ float ys[TV_B], rinv[TV_B];
  __shared__ float part[8][TV_B];
  __shared__ float xs[2][TV_B];
  __shared__ int s_b, s_fail;
  const int nb = (n + TV_B - 1) / TV_B;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    const int t = atomicAdd(ticket, 1);
    s_b = lower ? t : nb - 1 - t;
    s_fail = 0;
  }
  __syncthreads();
  const int b = s_b;
  const int r0 = b * TV_B;
  const int nr = (n - r0 < TV_B) ? n - r0 : TV_B;
  for (int e = threadIdx.x; e < nr * nr; e += 256) {
    const int i = e % nr, k = e / nr;
    tri[i][k] = A[(r0 + i) + (size_t)(r0 + k) * lda];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += 256) rinv[i] = unit ? 1.0f : 1.0f / tri[i][i];
  __syncthreads();
  {   // inverse of the diagonal block, one thread per column, while earlier blocks solve
    const int j = threadIdx.x;
    if (j < TV_B) {
      for (int i = 0; i < TV_B; ++i) tinv[i][j] = 0.0f;
      if (j < nr) {
        tinv[j][j] = rinv[j];
        if (lower) {
          for (int i = j + 1; i < nr; ++i) {
            float s = 0.0f;
            for (int k = j; k < i; ++k) s = fmaf(tri[i][k], tinv[k][j], s);
            tinv[i][j] = -s * rinv[i];
          }
        } else {
          for (int i = j - 1; i >= 0; --i) {
            float s = 0.0f;
            for (int k = i + 1; k <= j; ++k) s = fmaf(tri[i][k], tinv[k][j], s);
            tinv[i][j] = -s * rinv[i];
          }
        }
      }
    }
  }
  const float rhs0 = (w == 0 && lane < nr) ? x[r0 + lane] : 0.0f;          // own block: not written by others
  const float rhs1 = (w == 0 && lane + 32 < nr) ? x[r0 + lane + 32] : 0.0f;
  float acc0 = 0.0f, acc1 = 0.0f;
  for (int s = 0; s < nb - 1; ++s) {
    const int c = lower ? s : nb - 1 - s;
    if (lower ? c >= b : c <= b) break;
    const int c0 = c * TV_B;
    const int nc = (n - c0 < TV_B) ? n - c0 : TV_B;
    const int par = s & 1;
    float pa[16];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int k = w + 8 * m;
      const float *col = A + r0 + (size_t)(c0 + k) * lda;
      pa[2 * m] = (k < nc && lane < nr) ? col[lane] : 0.0f;
      pa[2 * m + 1] = (k < nc && lane + 32 < nr) ? col[lane + 32] : 0.0f;
    }
    if (threadIdx.x < nc) {
      const volatile unsigned long long *src = pub + c0 + threadIdx.x;
      unsigned i = 0;
      unsigned long long v = *src;
      while ((unsigned)(v >> 32) != epoch) {
        if (++i > kFlagPollLimit) { atomicOr(&g_trsv_status, kErrGridTimeout); s_fail = 1; break; }
        if (i > 32) __nanosleep(32);
        v = *src;
      }
      xs[par][threadIdx.x] = __uint_as_float((unsigned)(v & 0xffffffffull));
    }
    __syncthreads();
    if (s_fail) return;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int k = w + 8 * m;
      const float xk = (k < nc) ? xs[par][k] : 0.0f;
      acc0 = fmaf(pa[2 * m], xk, acc0);
      acc1 = fmaf(pa[2 * m + 1], xk, acc1);
    }
  }
  part[w][lane] = acc0;
  part[w][lane + 32] = acc1;
  __syncthreads();
  if (w == 0) {
    float y0 = 0.0f, y1 = 0.0f;
    for (int q = 0; q < 8; ++q) { y0 += part[q][lane]; y1 += part[q][lane + 32]; }
    ys[lane] = lane < nr ? rhs0 - y0 : 0.0f;
    ys[lane + 32] = lane + 32 < nr ? rhs1 - y1 : 0.0f;
  }
  __syncthreads();
  const int i = threadIdx.x >> 2, q = threadIdx.x & 3;
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 16; ++k) s = fmaf(tinv[i][q * 16 + k], ys[q * 16 + k], s);
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  if (q == 0 && i < nr) {
    x[r0 + i] = s;
    pub[r0 + i] = ((unsigned long long)epoch << 32) | (unsigned long long)__float_as_uint(s);
  }
}

static unsigned long long *trsv_pub_words(int n, unsigned *epoch, cudaStream_t st);

// op(A) x = x for one right-hand side (incx = 1), cblas Uplo/Trans/Diag.
template <typename T>
static void trsv_impl(int uplo, int tA, int diag, int n, const T *A, int lda, T *x, cudaStream_t st,
                      bool inv = false) {
  if (n <= 0) return;
  const int ta = (tA == kNoTrans) ? kNoTrans : kTrans;
  const int lower = ((uplo == kLower) != (ta != kNoTrans)) ? 1 : 0;
  const int nb = (n + TV_B - 1) / TV_B;
  int *w = static_cast<int *>(ctx().buffer(kBufV0, sizeof(int) * (size_t)(nb + 32)));
  ATLG_CHECK(cudaMemsetAsync(w, 0, sizeof(int) * (size_t)(nb + 32), st));
  if (inv && sizeof(T) == 4)   // FP32 only: the FP64 tiles would exceed static shared memory
    trsv_lookback_kernel<T, sizeof(T) == 4><<<nb, 256, 0, st>>>(n, A, lda, ta, lower, diag == kUnit ? 1 : 0, x,
                                                                w + 32, w);
  else
    trsv_lookback_kernel<T, false><<<nb, 256, 0, st>>>(n, A, lda, ta, lower, diag == kUnit ? 1 : 0, x, w + 32, w);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

void dev_dtrsv(int uplo, int ta, int diag, int n, const double *A, int lda, double *x, cudaStream_t st) {
  trsv_impl<double>(uplo, ta, diag, n, A, lda, x, st);
}
void dev_strsv(int uplo, int ta, int diag, int n, const float *A, int lda, float *x, cudaStream_t st) {
  trsv_impl<float>(uplo, ta, diag, n, A, lda, x, st);
}
void dev_strsv_inv(int uplo, int ta, int diag, int n, const float *A, int lda, float *x, cudaStream_t st) {
  if (n <= 0) return;
  if (ta != kNoTrans) {
    trsv_impl<float>(uplo, ta, diag, n, A, lda, x, st, true);
    return;
  }
  const int nb = (n + TV_B - 1) / TV_B;
  int *tk = static_cast<int *>(ctx().buffer(kBufV0, sizeof(int) * (size_t)(nb + 32)));
  unsigned epoch = 0;
  unsigned long long *pub = trsv_pub_words(n, &epoch, st);
  ATLG_CHECK(cudaMemsetAsync(tk, 0, sizeof(int), st));
  trsv_tagged_kernel<<<nb, 256, 0, st>>>(n, A, lda, uplo == kLower ? 1 : 0, diag == kUnit ? 1 : 0, x, pub, epoch,
                                         tk);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

// ------------------------------------------------------------ chained TRSV
// The mixed solver solves with one pair of FP32 triangular factors for up to
// 30 right-hand sides in a row.  trsv_chain_prep_kernel forms, once per
// factorization and for every 128-row block b of a triangle T, the inverse of
// its diagonal block Inv_b = T_bb^-1 and its coupling M_b = Inv_b T_bp to the
// block p solved just before it (p = b-1 for a lower triangle, b+1 for an
// upper one).  trsv_chain_kernel then solves with one CTA per block, blocks
// taken in solve order from an atomic ticket.  While the chain advances, a
// CTA streams the blocks solved two or more steps earlier and forms
// z_b = Inv_b (x_b - sum_c T_bc x_c); when x_p is published its own step is
// x_b = z_b - M_b x_p, one 128 x 128 product from shared memory.  Published
// values are 64-bit words (float value, call epoch), polled directly, so a
// value arrives with its signal.  A CTA only waits on blocks whose tickets
// were taken before its own; every wait is bounded.
constexpr int TC_B = 128;                  // rows per block
constexpr int TC_T = 512;                  // threads per CTA
constexpr int TC_LD = 132;                 // shared row stride: four 32-float quarters, each padded by one
constexpr size_t kChainPrepSmem = sizeof(float) * 3 * TC_B * (TC_B + 1);
constexpr size_t kChainSmem = sizeof(float) * 2 * TC_B * TC_LD;

__global__ void __launch_bounds__(TC_T)
    trsv_chain_prep_kernel(int n, const float *__restrict__ A, int lda, int lower, int unit, float *ws) {
  extern __shared__ float sm[];
  float *tri = sm;                         // [128][129]: the diagonal block
  float *inv = tri + TC_B * (TC_B + 1);    // [128][129]: its inverse
  float *cpl = inv + TC_B * (TC_B + 1);    // [128][129]: the coupling block T_bp
  __shared__ float rinv[TC_B];
  constexpr int L = TC_B + 1;
  const int nb = (n + TC_B - 1) / TC_B;
  const int b = blockIdx.x;
  const int r0 = b * TC_B, nr = min(TC_B, n - r0);
  const int p = lower ? b - 1 : b + 1;
  const int c0 = p * TC_B, nc = (p >= 0 && p < nb) ? min(TC_B, n - c0) : 0;
  for (int e = threadIdx.x; e < TC_B * TC_B; e += TC_T) {
    const int i = e % TC_B, k = e / TC_B;
    tri[i * L + k] = (i < nr && k < nr) ? A[(r0 + i) + (size_t)(r0 + k) * lda] : 0.0f;
    cpl[i * L + k] = (i < nr && k < nc) ? A[(r0 + i) + (size_t)(c0 + k) * lda] : 0.0f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < TC_B; i += TC_T) rinv[i] = (i < nr) ? (unit ? 1.0f : 1.0f / tri[i * L + i]) : 0.0f;
  __syncthreads();
  if (threadIdx.x < TC_B) {   // column j of the inverse by substitution, four partial sums
    const int j = threadIdx.x;
    for (int i = 0; i < TC_B; ++i) inv[i * L + j] = 0.0f;
    if (j < nr) {
      inv[j * L + j] = rinv[j];
      if (lower) {
        for (int i = j + 1; i < nr; ++i) {
          float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
          int k = j;
          for (; k + 3 < i; k += 4) {
            s0 = fmaf(tri[i * L + k], inv[k * L + j], s0);
            s1 = fmaf(tri[i * L + k + 1], inv[(k + 1) * L + j], s1);
            s2 = fmaf(tri[i * L + k + 2], inv[(k + 2) * L + j], s2);
            s3 = fmaf(tri[i * L + k + 3], inv[(k + 3) * L + j], s3);
          }
          for (; k < i; ++k) s0 = fmaf(tri[i * L + k], inv[k * L + j], s0);
          inv[i * L + j] = -((s0 + s1) + (s2 + s3)) * rinv[i];
        }
      } else {
        for (int i = j - 1; i >= 0; --i) {
          float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
          int k = i + 1;
          for (; k + 3 <= j; k += 4) {
            s0 = fmaf(tri[i * L + k], inv[k * L + j], s0);
            s1 = fmaf(tri[i * L + k + 1], inv[(k + 1) * L + j], s1);
            s2 = fmaf(tri[i * L + k + 2], inv[(k + 2) * L + j], s2);
            s3 = fmaf(tri[i * L + k + 3], inv[(k + 3) * L + j], s3);
          }
          for (; k <= j; ++k) s0 = fmaf(tri[i * L + k], inv[k * L + j], s0);
          inv[i * L + j] = -((s0 + s1) + (s2 + s3)) * rinv[i];
        }
      }
    }
  }
  __syncthreads();
  // row-major Inv_b, then M_b = Inv_b T_bp (zero where the block is ragged or absent)
  float *wi = ws + (size_t)b * 2 * TC_B * TC_B;
  float *wm = wi + TC_B * TC_B;
  for (int e = threadIdx.x; e < TC_B * TC_B; e += TC_T) wi[e] = inv[(e / TC_B) * L + (e % TC_B)];
  for (int e = threadIdx.x; e < TC_B * TC_B; e += TC_T) {
    const int i = e / TC_B, k = e % TC_B;
    float s0 = 0.0f, s1 = 0.0f;
    for (int j = 0; j < TC_B; j += 2) {
      s0 = fmaf(inv[i * L + j], cpl[j * L + k], s0);
      s1 = fmaf(inv[i * L + j + 1], cpl[(j + 1) * L + k], s1);
    }
    wm[e] = s0 + s1;
  }
}

// Waits until the 32 published words pub[0..31] (those with index < lim)
// carry `epoch` and returns in *v the float of word `lane` (0 past lim): the
// warp reads the 32 words with one coalesced load per lane per poll, and the
// callers broadcast them by shuffles (32 separate loads per lane of one word
// each, as in a per-thread loop, serialise on the volatile accesses).  With
// ns > 0, lane 0 first waits on word 0 alone, sleeping ns between polls, so
// that the many warps waiting on a block not yet solved poll cheaply.
// Returns false when the bounded wait gave up or another warp of the CTA
// already did (then *v = 0).
__device__ __forceinline__ bool chain_wait32(const unsigned long long *pub, int lim, unsigned epoch, float *v,
                                             volatile int *fail, unsigned ns) {
  const volatile unsigned long long *src = pub;
  const int lane = threadIdx.x & 31;
  unsigned tries = 0;
  int ok = 1;
  if (ns) {
    if (lane == 0 && lim > 0) {
      while ((unsigned)(src[0] >> 32) != epoch) {
        if (*fail) {
          ok = 0;
          break;
        }
        if (++tries > kFlagPollLimit) {
          atomicOr(&g_trsv_status, kErrGridTimeout);
          *fail = 1;
          ok = 0;
          break;
        }
        __nanosleep(ns);
      }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    tries = 0;
  }
  float val = 0.0f;
  while (ok) {
    bool mine = true;
    if (lane < lim) {
      const unsigned long long w = src[lane];
      val = __uint_as_float((unsigned)(w & 0xffffffffull));
      mine = (unsigned)(w >> 32) == epoch;
    }
    if (__all_sync(0xffffffffu, mine)) break;
    if (*fail) {
      ok = 0;
      break;
    }
    if (++tries > kFlagPollLimit) {
      if (lane == 0) atomicOr(&g_trsv_status, kErrGridTimeout);
      *fail = 1;
      ok = 0;
      break;
    }
    if (tries > 8) __nanosleep(32);
  }
  *v = ok ? val : 0.0f;
  return ok != 0;
}

__device__ __forceinline__ void chain_load32(const float *__restrict__ A, int lda, int n, int r0, int ri, int nr, int c0,
                                             int kq, float *dst) {
  const int nc = min(TC_B, n - c0);
  const float *col = A + (r0 + ri) + (size_t)(c0 + kq * 32) * lda;
#pragma unroll
  for (int k = 0; k < 32; ++k) dst[k] = (ri < nr && kq * 32 + k < nc) ? __ldcs(col + (size_t)k * lda) : 0.0f;
}

__global__ void __launch_bounds__(TC_T, 1)
    trsv_chain_kernel(int n, const float *__restrict__ A, int lda, int lower, const float *__restrict__ ws, float *x,
                      unsigned long long *pub, unsigned epoch, int *ticket) {
  extern __shared__ float sm[];
  float *sinv = sm;                        // [128][TC_LD] Inv_b, quarter-padded rows
  float *smc = sm + TC_B * TC_LD;          // [128][TC_LD] M_b
  __shared__ float part[4][TC_B];
  __shared__ float ys[4 * 33];             // quarter-padded
  __shared__ float xs[4 * 33];             // x of the block solved just before, quarter-padded
  __shared__ int s_pos;
  __shared__ volatile int s_fail;
  const int nb = (n + TC_B - 1) / TC_B;
  if (threadIdx.x == 0) {
    s_pos = atomicAdd(ticket, 1);
    s_fail = 0;
  }
  __syncthreads();
  const int pos = s_pos;                   // position in solve order
  const int b = lower ? pos : nb - 1 - pos;
  const int r0 = b * TC_B, nr = min(TC_B, n - r0);
  // stage Inv_b and M_b
  {
    const float4 *w4 = reinterpret_cast<const float4 *>(ws + (size_t)b * 2 * TC_B * TC_B);
    for (int e = threadIdx.x; e < 2 * TC_B * TC_B / 4; e += TC_T) {
      const int m = e / (TC_B * TC_B / 4);
      const int f = (e % (TC_B * TC_B / 4)) * 4;
      const int i = f / TC_B, k = f % TC_B;
      const float4 v = __ldg(w4 + e);
      float *d = (m ? smc : sinv) + i * TC_LD + (k >> 5) * 33 + (k & 31);
      d[0] = v.x;
      d[1] = v.y;
      d[2] = v.z;
      d[3] = v.w;
    }
  }
  // stream phase: blocks at solve positions 0 .. pos-2, rows ri, columns kq*32..kq*32+31
  const int ri = threadIdx.x & (TC_B - 1), kq = threadIdx.x >> 7;
  const float rhs = (threadIdx.x < TC_B && ri < nr) ? x[r0 + ri] : 0.0f;   // own rows: written only by this CTA
  float acc = 0.0f;
  const int nstream = pos - 1;
  if (nstream > 0) {
    // (a warp's lanes share kq: the 32 words of its quarter, one per lane)
    float pa[32], pb[32], xl;
    auto blk = [&](int q) { return lower ? q : nb - 1 - q; };
    auto fold = [&](const float *c) {
      float t = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) t = fmaf(c[k], __shfl_sync(0xffffffffu, xl, k), t);
      acc += t;
    };
    chain_load32(A, lda, n, r0, ri, nr, blk(0) * TC_B, kq, pa);
    for (int q = 0; q < nstream; q += 2) {
      if (q + 1 < nstream) chain_load32(A, lda, n, r0, ri, nr, blk(q + 1) * TC_B, kq, pb);
      {
        const int c0 = blk(q) * TC_B;
        chain_wait32(pub + c0 + kq * 32, min(TC_B, n - c0) - kq * 32, epoch, &xl, &s_fail, 128);
        fold(pa);
      }
      if (q + 1 >= nstream) break;
      if (q + 2 < nstream) chain_load32(A, lda, n, r0, ri, nr, blk(q + 2) * TC_B, kq, pa);
      {
        const int c0 = blk(q + 1) * TC_B;
        chain_wait32(pub + c0 + kq * 32, min(TC_B, n - c0) - kq * 32, epoch, &xl, &s_fail, 128);
        fold(pb);
      }
    }
  }
  part[kq][ri] = acc;
  __syncthreads();
  if (threadIdx.x < TC_B)
    ys[(ri >> 5) * 33 + (ri & 31)] = rhs - ((part[0][ri] + part[1][ri]) + (part[2][ri] + part[3][ri]));
  __syncthreads();
  // (after a wait that gave up the block is still published, with the status
  // bit set, so that later blocks do not wait out their own limits)
  // z = Inv_b y: four threads per row, 32 terms each
  const int hi = threadIdx.x >> 2, hq = threadIdx.x & 3;
  float z = 0.0f;
  {
    const float *irow = sinv + hi * TC_LD + hq * 33;
    const float *yq = ys + hq * 33;
#pragma unroll
    for (int k = 0; k < 32; ++k) z = fmaf(irow[k], yq[k], z);
    z += __shfl_xor_sync(0xffffffffu, z, 1);
    z += __shfl_xor_sync(0xffffffffu, z, 2);
  }
  // the hop: x_b = z - M_b x_p; warps 0-3 wait for x_p, a quarter each, and
  // stage it in shared memory
  if (pos > 0) {
    const int c0 = (lower ? b - 1 : b + 1) * TC_B;
    float mrow[32], t = 0.0f;
#pragma unroll
    for (int k = 0; k < 32; ++k) mrow[k] = smc[hi * TC_LD + hq * 33 + k];
    const int w = threadIdx.x >> 5;
    if (w < 4) {
      float xl;
      chain_wait32(pub + c0 + w * 32, min(TC_B, n - c0) - w * 32, epoch, &xl, &s_fail, 0);
      xs[w * 33 + (threadIdx.x & 31)] = xl;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 32; ++k) t = fmaf(mrow[k], xs[hq * 33 + k], t);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    z -= t;
  }
  if (hq == 0 && hi < nr) {
    x[r0 + hi] = z;
    pub[r0 + hi] = ((unsigned long long)epoch << 32) | (unsigned long long)__float_as_uint(z);
  }
}

// The published-word buffer shared by the tagged and chained TRSV: zeroed
// whenever it is new, epochs counting from 1.
static unsigned long long *trsv_pub_words(int n, unsigned *epoch, cudaStream_t st) {
  static unsigned long long *s_pub = nullptr;
  static size_t s_len = 0;
  static unsigned s_epoch = 0;
  unsigned long long *pub =
      static_cast<unsigned long long *>(ctx().buffer(kBufV2, sizeof(unsigned long long) * (size_t)n));
  if (pub != s_pub || (size_t)n > s_len || s_epoch == 0xffffffffu) {
    ATLG_CHECK(cudaMemsetAsync(pub, 0, sizeof(unsigned long long) * (size_t)n, st));
    s_pub = pub;
    s_len = (size_t)n > s_len ? (size_t)n : s_len;
    s_epoch = 0;
  }
  *epoch = ++s_epoch;
  return pub;
}

size_t strsv_chain_ws_floats(int n) { return (size_t)((n + TC_B - 1) / TC_B) * 2 * TC_B * TC_B; }

void dev_strsv_chain_prepare(int uplo, int diag, int n, const float *A, int lda, float *ws, cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    ATLG_CHECK(cudaFuncSetAttribute(trsv_chain_prep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kChainPrepSmem));
    ATLG_CHECK(cudaFuncSetAttribute(trsv_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kChainSmem));
    attr = true;
  }
  const int nb = (n + TC_B - 1) / TC_B;
  trsv_chain_prep_kernel<<<nb, TC_T, kChainPrepSmem, st>>>(n, A, lda, uplo == kLower ? 1 : 0, diag == kUnit ? 1 : 0,
                                                           ws);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

void dev_strsv_chain(int uplo, int n, const float *A, int lda, const float *ws, float *x, cudaStream_t st) {
  if (n <= 0) return;
  const int nb = (n + TC_B - 1) / TC_B;
  unsigned epoch = 0;
  unsigned long long *pub = trsv_pub_words(n, &epoch, st);
  int *tk = static_cast<int *>(ctx().buffer(kBufV0, sizeof(int) * (size_t)(nb + 32)));
  ATLG_CHECK(cudaMemsetAsync(tk, 0, sizeof(int), st));
  trsv_chain_kernel<<<nb, TC_T, kChainSmem, st>>>(n, A, lda, uplo == kLower ? 1 : 0, ws, x, pub, epoch, tk);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

unsigned trsv_status_read_and_clear() {
  unsigned v = 0, z = 0;
  ATLG_CHECK(cudaMemcpyFromSymbol(&v, g_trsv_status, sizeof(v)));
  if (v) ATLG_CHECK(cudaMemcpyToSymbol(g_trsv_status, &z, sizeof(z)));
  return v;
}

}  // namespace atlg
