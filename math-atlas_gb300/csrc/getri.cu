// getri.cu -- triangular inverse and the inverse from LU factors on GB300:
// clapack_?trtri and clapack_?getri, FP64 and FP32.
//
// Reference path replaced: ATL_trtri with the recursive ATL_trtriCU/CL/RU/RL
// (AtlasBase/Clint/atlas-lp.base:1718-2380) and ATL_getriC/getriR with
// clapack_getri (atlas-lp.base:16-220, AtlasBase/Clint/atlas-clp.base:115-139).
//
// GB300 design.
//  * trtri keeps the reference's recursive split (the off-diagonal block of
//    each split becomes -inv(A11) A12 inv(A22)) at multiples of 64, but runs
//    it bottom-up: one launch inverts every 64 x 64 diagonal block (one CTA
//    each, in shared memory), then each split, children first, forms its
//    off-diagonal block from the two inverses already in place with GEMMs
//    whose triangular operand skips the zero k-tiles -- no triangular solves,
//    whose short dependency chains left the FP64 pipe idle.
//  * getri: inv(U) by trtri, the strictly lower factor moved to a workspace
//    (zeros left in A) by one kernel, X L = inv(U) as a single Right/Lower/
//    Unit TRSM over the whole matrix, and the column interchanges composed on
//    the host into one permutation applied by a gather kernel.
//  * A zero on a non-unit diagonal is found by one reduction kernel before
//    anything is written, as ATL_trtri checks first and returns its index.
//  * RowMajor data: the row-major inverse of one triangle is the column-major
//    inverse of the other on the same memory, and row-major getri is
//    column-major getri on the same memory and pivots.
#include <limits.h>

#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "getri.cuh"
#include "trsm.cuh"

namespace atlg {

constexpr int TB = 64;

template <typename T>
__global__ void diag_zero_kernel(int n, const T *A, int lda, int *first) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (A[i + (size_t)i * lda] == T(0)) atomicMin(first, i);
}

// Invert every diagonal block (64 x 64, the last one smaller) of an upper
// (upper != 0) or lower triangular matrix in place; one CTA per block.  The
// lower case works on the transpose (inv(L)^T = inv(L^T)).  Column j of the
// inverse: x = inv(U(0:j,0:j)) * U(0:j,j) scaled by -1/U(j,j), the columns
// before j already inverted in shared memory.
template <typename T>
__global__ void __launch_bounds__(64) trtri_leaf_kernel(int n, int upper, int unit, T *A, int lda) {
  __shared__ T a[TB][TB + 1];
  const int o = blockIdx.x * TB;
  const int nb = (n - o < TB) ? n - o : TB;
  const int tid = threadIdx.x;
  T *Ab = A + o + (size_t)o * lda;
  for (int e = tid; e < nb * nb; e += TB) {
    const int i = e % nb, k = e / nb;
    if (i <= k) a[i][k] = upper ? Ab[i + (size_t)k * lda] : Ab[k + (size_t)i * lda];
  }
  __syncthreads();
  if (unit && tid < nb) a[tid][tid] = T(1);
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const T dinv = unit ? T(1) : T(1) / a[j][j];
    T t = T(0);
    if (tid < j)
      for (int k = tid; k < j; ++k) t += a[tid][k] * a[k][j];
    __syncthreads();
    if (tid < j) a[tid][j] = -dinv * t;
    if (tid == j) a[j][j] = dinv;
    __syncthreads();
  }
  for (int e = tid; e < nb * nb; e += TB) {
    const int i = e % nb, k = e / nb;
    if (i > k || (unit && i == k)) continue;
    if (upper) Ab[i + (size_t)k * lda] = a[i][k];
    else Ab[k + (size_t)i * lda] = a[i][k];
  }
}

template <typename T>
static void trsm_t(int side, int uplo, int diag, int M, int N, T alpha, const T *A, int lda, T *B, int ldb,
                   cudaStream_t st) {
  if (sizeof(T) == 8)
    dev_dtrsm(side, uplo, kNoTrans, diag, M, N, (double)alpha, (const double *)A, lda, (double *)B, ldb, st);
  else
    dev_strsm(side, uplo, kNoTrans, diag, M, N, (float)alpha, (const float *)A, lda, (float *)B, ldb, st);
}

template <typename T>
static void gemm_t(int M, int N, int K, T alpha, const T *A, int lda, const T *B, int ldb, T beta, T *C, int ldc,
                   int tri, cudaStream_t st, int batch = 1, long sa = 0, long sb = 0, long sc = 0) {
  if (M <= 0 || N <= 0 || K <= 0 || batch <= 0) return;
  GemmOpts o;
  o.tri = tri;
  o.batch = batch;
  o.stride_a = sa;
  o.stride_b = sb;
  o.stride_c = sc;
  if (sizeof(T) == 8)
    dev_dgemm(kNoTrans, kNoTrans, M, N, K, (double)alpha, (const double *)A, lda, (const double *)B, ldb,
              (double)beta, (double *)C, ldc, st, o);
  else
    dev_sgemm(kNoTrans, kNoTrans, M, N, K, (float)alpha, (const float *)A, lda, (const float *)B, ldb, (float)beta,
              (float *)C, ldc, st, o);
}

// Columns of the off-diagonal block computed per pass (bounds the workspace).
constexpr int kTriChunk = 1024;

// One split of the recursion whose diagonal blocks already hold their
// inverses X11 (nl x nl at P) and X22 (nr x nr):
//   lower:  X21 = -X22 (L21 X11),   upper:  X12 = -X11 (U12 X22),
// as GEMMs whose triangular operand skips the k-tiles outside its triangle.
// The inner product goes through a workspace W of at most kTriChunk columns:
// columns [c0, c1) of L21 X11 are L21(:, c0:c1) X11(c0:c1, c0:c1) (lower
// triangular operand) + L21(:, c1:) X11(c1:, c0:c1) (dense), so the chunks
// run left to right and overwrite L21 in place; those of U12 X22 are
// U12(:, c0:c1) X22(c0:c1, c0:c1) (upper) + U12(:, :c0) X22(:c0, c0:c1),
// right to left.
template <typename T>
static void combine_node(int upper, int unit, int nl, int nr, T *P, int lda, T *W, cudaStream_t st) {
  T *A22 = P + nl + (size_t)nl * lda;
  if (!upper) {
    T *A21 = P + nl;                                           // nr x nl
    for (int c0 = 0; c0 < nl; c0 += kTriChunk) {
      const int c1 = (c0 + kTriChunk < nl) ? c0 + kTriChunk : nl, w = c1 - c0;
      const T *X11c = P + c0 + (size_t)c0 * lda;               // X11(c0:, c0:c1)
      gemm_t<T>(nr, w, w, T(1), A21 + (size_t)c0 * lda, lda, X11c, lda, T(0), W, nr, kTriB | unit, st);
      gemm_t<T>(nr, w, nl - c1, T(1), A21 + (size_t)c1 * lda, lda, X11c + w, lda, T(1), W, nr, 0, st);
      gemm_t<T>(nr, w, nr, T(-1), A22, lda, W, nr, T(0), A21 + (size_t)c0 * lda, lda, kTriA | unit, st);
    }
  } else {
    T *A12 = P + (size_t)nl * lda;                             // nl x nr
    for (int c1 = nr; c1 > 0; c1 -= kTriChunk) {
      const int c0 = (c1 - kTriChunk > 0) ? c1 - kTriChunk : 0, w = c1 - c0;
      const T *X22c = A22 + (size_t)c0 * lda;                  // X22(:, c0:c1)
      gemm_t<T>(nl, w, w, T(1), A12 + (size_t)c0 * lda, lda, X22c + c0, lda, T(0), W, nl,
                kTriB | kTriUpper | unit, st);
      gemm_t<T>(nl, w, c0, T(1), A12, lda, X22c, lda, T(1), W, nl, 0, st);
      gemm_t<T>(nl, w, nl, T(-1), P, lda, W, nl, T(0), A12 + (size_t)c0 * lda, lda, kTriA | kTriUpper | unit, st);
    }
  }
}

// Bottom-up recursion over aligned power-of-two blocks: after the 64 x 64
// diagonal blocks are inverted, level b (64, 128, ...) combines every
// aligned 2b block [2bz, 2bz + 2b) from its two inverted halves; the full
// blocks of a level go in one batched GEMM per step (when one chunk covers
// them), a ragged last block (second half shorter than b) on its own.
template <typename T>
static void trtri_combine(int upper, int diag, int n, T *A, int lda, T *W, cudaStream_t st) {
  const int unit = (diag == kUnit) ? kTriUnit : 0;
  for (int b = TB; b < n; b *= 2) {
    const int count = n / (2 * b);
    const long sd = 2L * b * (lda + 1);                        // diagonal step between blocks
    if (count > 0 && b <= kTriChunk) {
      const long sw = (long)b * b;
      if (!upper) {
        // W_z = L21_z X11_z;  L21_z = -X22_z W_z
        gemm_t<T>(b, b, b, T(1), A + b, lda, A, lda, T(0), W, b, kTriB | unit, st, count, sd, sd, sw);
        gemm_t<T>(b, b, b, T(-1), A + b + (size_t)b * lda, lda, W, b, T(0), A + b, lda, kTriA | unit, st, count, sd,
                  sw, sd);
      } else {
        // W_z = U12_z X22_z;  U12_z = -X11_z W_z
        gemm_t<T>(b, b, b, T(1), A + (size_t)b * lda, lda, A + b + (size_t)b * lda, lda, T(0), W, b,
                  kTriB | kTriUpper | unit, st, count, sd, sd, sw);
        gemm_t<T>(b, b, b, T(-1), A, lda, W, b, T(0), A + (size_t)b * lda, lda, kTriA | kTriUpper | unit, st, count,
                  sd, sw, sd);
      }
    } else {
      for (int z = 0; z < count; ++z) combine_node<T>(upper, unit, b, b, A + z * sd, lda, W, st);
    }
    const int r0 = count * 2 * b;
    if (r0 + b < n) combine_node<T>(upper, unit, b, n - r0 - b, A + (size_t)r0 * (lda + 1), lda, W, st);
  }
}

// Column-major inverse of the `upper` triangle in place; 0 or the 1-based
// index of the first zero on a non-unit diagonal (A untouched then).
template <typename T>
static int trtri_impl(int upper, int diag, int n, T *A, int lda, cudaStream_t st) {
  if (n <= 0) return 0;
  if (diag != kUnit) {
    int *d = static_cast<int *>(ctx().buffer(kBufChol, 64));
    ATLG_CHECK(cudaMemsetAsync(d, 0x7f, sizeof(int), st));
    int blocks = (n + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    diag_zero_kernel<T><<<blocks, 256, 0, st>>>(n, A, lda, d);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    int first = INT_MAX;
    ATLG_CHECK(cudaMemcpyAsync(&first, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    ATLG_CHECK(cudaStreamSynchronize(st));
    if (first < n) return first + 1;
  }
  trtri_leaf_kernel<T><<<(n + TB - 1) / TB, TB, 0, st>>>(n, upper, diag == kUnit ? 1 : 0, A, lda);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
  if (n > TB) {
    // workspace: a level's batched products (count * b * b <= n * b / 2 for
    // b <= kTriChunk) or one node's chunk (at most n/2 x kTriChunk)
    size_t welems = 0;
    for (int b = TB; b < n; b *= 2) {
      const size_t need = (b <= kTriChunk) ? (size_t)(n / (2 * b)) * b * b + (size_t)b * b
                                           : (size_t)b * kTriChunk;
      if (need > welems) welems = need;
    }
    T *W = static_cast<T *>(ctx().buffer(kBufTri, sizeof(T) * welems));
    trtri_combine<T>(upper, diag, n, A, lda, W, st);
  }
  return 0;
}

int dev_dtrtri(int order, int uplo, int diag, int n, double *A, int lda, cudaStream_t st) {
  const int upper = (uplo == kUpper) == (order == kColMajor);
  return trtri_impl<double>(upper, diag, n, A, lda, st);
}
int dev_strtri(int order, int uplo, int diag, int n, float *A, int lda, cudaStream_t st) {
  const int upper = (uplo == kUpper) == (order == kColMajor);
  return trtri_impl<float>(upper, diag, n, A, lda, st);
}

// W(i,j) = A(i,j), A(i,j) = 0 for i > j (the unit-lower factor leaves A).
template <typename T>
__global__ void split_lower_kernel(int n, T *A, int lda, T *W, int ldw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int j = blockIdx.y; j < n; j += gridDim.y) {
    if (i > j && i < n) {
      T *a = A + i + (size_t)j * lda;
      W[i + (size_t)j * ldw] = *a;
      *a = T(0);
    }
  }
}

// W(:, c) = A(:, perm[c])
template <typename T>
__global__ void gather_cols_kernel(int n, const T *A, int lda, const int *perm, T *W, int ldw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int c = blockIdx.y; c < n; c += gridDim.y)
    if (i < n) W[i + (size_t)c * ldw] = A[i + (size_t)perm[c] * lda];
}

// Column-major inverse from getrf's factors and 0-based pivots (host array).
template <typename T>
static int getri_impl(int n, T *A, int lda, const int *ipiv_host, cudaStream_t st) {
  if (n <= 0) return 0;
  const int info = trtri_impl<T>(1, kNonUnit, n, A, lda, st);
  if (info || n < 2) return info;
  Context &c = ctx();
  const int ldw = (n + 1) & ~1;
  T *W = static_cast<T *>(c.buffer(kBufTrmm, sizeof(T) * (size_t)ldw * n));
  const dim3 grid((n + 255) / 256, n < 4096 ? n : 4096);
  split_lower_kernel<T><<<grid, 256, 0, st>>>(n, A, lda, W, ldw);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
  trsm_t<T>(kRight, kLower, kUnit, n, n, T(1), W, ldw, A, lda, st);   // X L = inv(U)
  // column interchanges J = n-2 .. 0, composed: column c of the result is
  // column perm[c] of X
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  bool any = false;
  for (int J = n - 2; J >= 0; --J) {
    const int jp = ipiv_host[J];
    if (jp != J) {
      const int t = perm[J]; perm[J] = perm[jp]; perm[jp] = t;
      any = true;
    }
  }
  if (any) {
    int *dperm = static_cast<int *>(c.buffer(kBufPiv, sizeof(int) * (size_t)n));
    ATLG_CHECK(cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    gather_cols_kernel<T><<<grid, 256, 0, st>>>(n, A, lda, dperm, W, ldw);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    ATLG_CHECK(cudaMemcpy2DAsync(A, sizeof(T) * lda, W, sizeof(T) * ldw, sizeof(T) * n, n, cudaMemcpyDeviceToDevice,
                                 st));
    // perm lives in pageable host memory: the copy is complete before
    // cudaMemcpyAsync returns, so the vector may go out of scope
  }
  return 0;
}

int dev_dgetri(int n, double *A, int lda, const int *ipiv_host, cudaStream_t st) {
  return getri_impl<double>(n, A, lda, ipiv_host, st);
}
int dev_sgetri(int n, float *A, int lda, const int *ipiv_host, cudaStream_t st) {
  return getri_impl<float>(n, A, lda, ipiv_host, st);
}

}  // namespace atlg
