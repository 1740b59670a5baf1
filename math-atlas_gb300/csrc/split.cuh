// split.cuh -- split-precision (integer-slice, tensor-core) DGEMM.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// C = alpha*op(A)*op(B) + beta*C, column-major FP64 on the device, computed
// from `nslices` (1..8) 7-bit slices per operand on tcgen05 tensor cores.
void dev_dgemm_split(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
                     int ldb, double beta, double *C, int ldc, int nslices, cudaStream_t st);
unsigned split_status_read_and_clear();

}  // namespace atlg
