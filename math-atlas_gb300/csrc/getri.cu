// getri.cu -- triangular inverse and the inverse from LU factors on GB300:
// clapack_?trtri and clapack_?getri, FP64 and FP32.
//
// Reference path replaced: ATL_trtri with the recursive ATL_trtriCU/CL/RU/RL
// (AtlasBase/Clint/atlas-lp.base:1718-2380) and ATL_getriC/getriR with
// clapack_getri (atlas-lp.base:16-220, AtlasBase/Clint/atlas-clp.base:115-139).
//
// GB300 design.
//  * trtri keeps the reference's recursion -- the off-diagonal block of each
//    split becomes -inv(A11) A12 inv(A22) through two TRSMs -- but splits at
//    multiples of 64 and defers the diagonal blocks: every TRSM reads only
//    original diagonal blocks, so all of them are issued first (pre-order),
//    and one launch then inverts every 64 x 64 diagonal block, one CTA each,
//    in shared memory.
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

// The off-diagonal blocks of the recursion, pre-order (diagonal blocks later).
template <typename T>
static void trtri_offdiag(int upper, int diag, int n, T *A, int lda, cudaStream_t st) {
  if (n <= TB) return;
  const int nl = ((n / 2 + TB - 1) / TB) * TB;
  const int nr = n - nl;
  T *A22 = A + nl + (size_t)nl * lda;
  if (upper) {
    T *A12 = A + (size_t)nl * lda;
    trsm_t<T>(kRight, kUpper, diag, nl, nr, T(1), A22, lda, A12, lda, st);   // A12 inv(U22)
    trsm_t<T>(kLeft, kUpper, diag, nl, nr, T(-1), A, lda, A12, lda, st);     // -inv(U11) A12 inv(U22)
  } else {
    T *A21 = A + nl;
    trsm_t<T>(kRight, kLower, diag, nr, nl, T(1), A, lda, A21, lda, st);     // A21 inv(L11)
    trsm_t<T>(kLeft, kLower, diag, nr, nl, T(-1), A22, lda, A21, lda, st);   // -inv(L22) A21 inv(L11)
  }
  trtri_offdiag<T>(upper, diag, nl, A, lda, st);
  trtri_offdiag<T>(upper, diag, nr, A22, lda, st);
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
  trtri_offdiag<T>(upper, diag, n, A, lda, st);
  trtri_leaf_kernel<T><<<(n + TB - 1) / TB, TB, 0, st>>>(n, upper, diag == kUnit ? 1 : 0, A, lda);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
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
