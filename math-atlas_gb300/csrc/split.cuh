// split.cuh -- split-precision (integer-slice, tensor-core) DGEMM.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace atlg {

// C = alpha*op(A)*op(B) + beta*C, column-major FP64 on the device, computed
// from `nslices` (1..8) 7-bit slices per operand on tcgen05 tensor cores.
void dev_dgemm_split(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
                     int ldb, double beta, double *C, int ldc, int nslices, cudaStream_t st);
// The same product in two steps, so one slicing can feed launches on several
// streams: prepare slices both operands (K <= 16384) into one of two sets of
// the library's split slots (one prepared product per set at a time; set 0
// is also the one dev_dgemm_split uses); run computes the output column tiles
// [t0, t1) (256 columns each).
struct SplitArgs {
  int M, N, Mp, Np, Kp, s;
  int nt0;                 // first output column tile of a launch
  double alpha, beta;
  int alpha_pow2, alpha_exp;   // alpha = +-2^alpha_exp exactly (integer-only scaling)
  double *C;
  int ldc;
  const int *exA, *exB;
};
struct SplitPlan {
  CUtensorMap tA, tB;
  SplitArgs a;
};
constexpr int kSplitTileN = 256;
void dev_dgemm_split_prepare(int TA, int TB, int M, int N, int K, const double *A, int lda, const double *B, int ldb,
                             int s, SplitPlan *plan, cudaStream_t st, int slot_set = 0);
void dev_dgemm_split_run(const SplitPlan &plan, int t0, int t1, double alpha, double beta, double *C, int ldc,
                         cudaStream_t st);
unsigned split_status_read_and_clear();

}  // namespace atlg
