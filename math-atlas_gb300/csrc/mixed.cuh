// mixed.cuh -- mixed-precision solve (FP32 LU + FP64 iterative refinement).
#pragma once
#include <cuda_runtime.h>
#include <vector>

namespace atlg {

struct MixedResult {
  int iters = 0;              // refinement steps taken
  int status = 0;             // 0: converged in mixed precision, 1: FP64 LU fallback, 2: singular
  std::vector<double> berr;   // per right-hand side: ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
  std::vector<double> ferr;   // per right-hand side: ||d||_inf / ||x||_inf of the last correction
};

// Device data, column-major.  A is unchanged unless the FP64 fallback ran
// (then it holds the FP64 factors); B is unchanged; X receives the solution.
int dev_dgesv_mixed(int n, int nrhs, double *A, int lda, int *ipiv, const double *B, int ldb, double *X, int ldx,
                    MixedResult *res, cudaStream_t st);
// Single right-hand side refinement solves: the chained 128-row TRSV (true)
// or the tagged 64-row look-back TRSV (false).
void set_refine_trsv_chained(bool on);
// SA = A in FP32, round to nearest even (LAPACK dlag2s); returns 1 when some
// |a| exceeds FLT_MAX, else 0.  Synchronizes the stream.
int dev_dlag2s(int M, int N, const double *A, int lda, float *SA, int ldsa, cudaStream_t st);

}  // namespace atlg
