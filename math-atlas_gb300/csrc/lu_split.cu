// lu_split.cu -- FP64 LU whose trailing updates run on the split-precision
// DGEMM (integer slices on tcgen05 tensor cores, split.cu): the "split-DGEMM
// form" of dgesv.  No reference counterpart: ATLAS has one LU, in FP64 on the
// FP64 pipe (ATL_getrfC, AtlasBase/Clint/atlas-lp.base:1210-1617); this
// factorization computes the same partial-pivoting LU with the O(n^3) part of
// the work moved to the tensor pipe.
//
// Outer blocks of nb columns (a multiple of 256; 1024 by default), right-
// looking, with look-ahead:
//  1. the (n-k) x nb block column is factored by this same method with
//     512-column blocks (split updates between them), each of those by the
//     FP64 LU (lu.cu: 32-wide panels, look-ahead, DFMA updates);
//  2. its interchanges are applied to the columns left and right of it;
//  3. U12 = L11^-1 A12 as inv(L11) (unit lower, trtri in FP64) times A12 on
//     the split DGEMM;
//  4. A22 -= L21 U12 on the split DGEMM with K = nb, sliced once: the next
//     block column's tiles on the caller's stream, the rest on a second
//     low-priority stream, so the FP64 factorization of the next block column
//     (FP64 pipe) overlaps the bulk of the update (tensor pipe); the next
//     interchanges wait for it.
// With 8 slices each split product is accurate to about 3e-16 of
// sum |a||b| (the FP64 GEMM's own error bound is of that order), so the
// factorization is FP64-accurate at any condition number.  Pivots can differ
// from the plain FP64 LU where two candidates are within rounding.
#include "common.cuh"
#include "context.cuh"
#include "getri.cuh"
#include "lu.cuh"
#include "lu_split.cuh"
#include "split.cuh"

namespace atlg {


__global__ void add_offset_kernel(int *ipiv, int n, int off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ipiv[i] += off;
}

// W = the unit lower triangle of the kb x kb block at A (zeros above).
__global__ void unit_lower_kernel(int kb, const double *A, int lda, double *W, int ldw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int j = blockIdx.y; j < kb; j += gridDim.y)
    if (i < kb) W[i + (size_t)j * ldw] = (i > j) ? A[i + (size_t)j * lda] : (i == j ? 1.0 : 0.0);
}

// Widest block column handed to the FP64 LU (a multiple of 256); wider ones
// are factored recursively with blocks of this width.  The leaves' FP64 LU
// uses 32-wide panels: a panel's own rank-1 updates run on the FP64 pipe of
// the few SMs the panel occupies, a narrower panel leaves more of that work
// to the leaf's DGEMMs on every SM.  Measured at n = 16384 with 1024-wide
// outer blocks: leaves 1024/512/256 with 64-wide panels 362/360/382 ms,
// 512-wide leaves with 32-wide panels 342 ms.
constexpr int kLeafDefault = 512, kLeafPanel = 32;
static int g_leaf_nb = kLeafDefault;
void set_split_lu_leaf(int nb) { g_leaf_nb = (nb >= kSplitTileN) ? nb / kSplitTileN * kSplitTileN : kLeafDefault; }

// M x N (M >= N) partial-pivoting LU of A in place; pivots relative to row 0
// of A; returns 0 or the first zero pivot (1-based).  Outer blocks of nb
// columns; a block column wider than g_leaf_nb is itself factored by this
// routine with g_leaf_nb blocks (no look-ahead there), a narrower one by the
// FP64 LU.  With lookahead, each trailing update is sliced once into the
// second slot set, its first block of columns is computed on st and the rest
// on the library's outer stream, overlapping the next block column.
static int split_lu(int M, int N, double *A, int lda, int *ipiv, int nslices, int nb, bool lookahead,
                    cudaStream_t st) {
  Context &c = ctx();
  const int NB2 = (nb >= kSplitTileN) ? (nb / kSplitTileN) * kSplitTileN : g_leaf_nb;
  int *dinfo = static_cast<int *>(c.buffer(kBufX2, 64));
  cudaStream_t outer = c.outer_stream();
  cudaEvent_t ev_ready = c.sync_event(2), ev_done = c.sync_event(3);
  bool outer_pending = false;
  int info = 0;
  for (int k = 0; k < N; k += NB2) {
    const int kb = (N - k < NB2) ? N - k : NB2;
    const int m = M - k, r = N - k - kb;
    double *Akk = A + k + (size_t)k * lda;
    int binfo = 0;
    bool leaf = kb <= g_leaf_nb;
    if (!leaf) {
      binfo = split_lu(m, kb, Akk, lda, ipiv + k, nslices, g_leaf_nb, false, st);   // relative to row k
    } else {
      dev_dgetrf_pw(m, kb, Akk, lda, ipiv + k, dinfo, kLeafPanel, st);        // relative to row k
      ATLG_CHECK(cudaMemcpyAsync(&binfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    if (outer_pending) {   // the interchanges touch every column
      ATLG_CHECK(cudaStreamWaitEvent(st, ev_done, 0));
      outer_pending = false;
    }
    // interchanges on the rows k.. of the columns left and right of the block
    if (k > 0) dev_dlaswp(k, A + k, lda, 0, kb, ipiv + k, 1, m, st);
    if (r > 0) dev_dlaswp(r, A + k + (size_t)(k + kb) * lda, lda, 0, kb, ipiv + k, 1, m, st);
    add_offset_kernel<<<(kb + 255) / 256, 256, 0, st>>>(ipiv + k, kb, k);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    if (leaf) ATLG_CHECK(cudaStreamSynchronize(st));   // binfo has arrived
    if (binfo > 0 && info == 0) info = k + binfo;
    if (r <= 0) continue;
    double *A12 = A + k + (size_t)(k + kb) * lda;
    double *A22 = A + (k + kb) + (size_t)(k + kb) * lda;
    // U12 = inv(L11) A12, through a workspace
    const int ldw = (kb + 1) & ~1;
    double *W = static_cast<double *>(c.buffer(kBufX0, sizeof(double) * (size_t)ldw * kb));
    double *T = static_cast<double *>(c.buffer(kBufX1, sizeof(double) * (size_t)ldw * r));
    unit_lower_kernel<<<dim3((kb + 255) / 256, kb), 256, 0, st>>>(kb, Akk, lda, W, ldw);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    dev_dtrtri(kColMajor, kLower, kUnit, kb, W, ldw, st);
    dev_dgemm_split(kNoTrans, kNoTrans, kb, r, kb, 1.0, W, ldw, A12, lda, 0.0, T, ldw, nslices, st);
    ATLG_CHECK(cudaMemcpy2DAsync(A12, sizeof(double) * lda, T, sizeof(double) * ldw, sizeof(double) * kb, r,
                                 cudaMemcpyDeviceToDevice, st));
    // A22 -= L21 U12
    if (!lookahead) {
      dev_dgemm_split(kNoTrans, kNoTrans, m - kb, r, kb, -1.0, Akk + kb, lda, A12, lda, 1.0, A22, lda, nslices, st);
      continue;
    }
    SplitPlan plan;
    dev_dgemm_split_prepare(kNoTrans, kNoTrans, m - kb, r, kb, Akk + kb, lda, A12, lda, nslices, &plan, st, 1);
    const int first = r < NB2 ? r : NB2;
    const int tnext = (first + kSplitTileN - 1) / kSplitTileN;
    dev_dgemm_split_run(plan, 0, tnext, -1.0, 1.0, A22, lda, st);
    const int tall = (r + kSplitTileN - 1) / kSplitTileN;
    if (tnext < tall) {
      ATLG_CHECK(cudaEventRecord(ev_ready, st));
      ATLG_CHECK(cudaStreamWaitEvent(outer, ev_ready, 0));
      dev_dgemm_split_run(plan, tnext, tall, -1.0, 1.0, A22, lda, outer);
      ATLG_CHECK(cudaEventRecord(ev_done, outer));
      outer_pending = true;
    }
  }
  if (outer_pending) ATLG_CHECK(cudaStreamWaitEvent(st, ev_done, 0));
  return info;
}

int dev_dgetrf_split(int n, double *A, int lda, int *ipiv, int nslices, int nb, cudaStream_t st) {
  if (n <= 0) return 0;
  return split_lu(n, n, A, lda, ipiv, nslices, nb, true, st);
}

}  // namespace atlg
