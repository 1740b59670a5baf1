// lu_split.cuh -- FP64 LU with split-precision (tensor-core) trailing updates.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// Column-major n x n partial-pivoting LU in place (0-based absolute pivots);
// returns 0 or the 1-based index of the first zero pivot.  nslices: 7-bit
// slices per operand of the split products (8 for FP64 accuracy); nb: the
// outer block width (rounded down to a multiple of 256; the K of the split
// products).
// Synchronizes once per outer block (the block column's info).
int dev_dgetrf_split(int n, double *A, int lda, int *ipiv, int nslices, int nb, cudaStream_t st);
// Widest block column factored by the FP64 LU inside the split LU (rounded
// down to a multiple of 256; below 256: the default 1024).
void set_split_lu_leaf(int nb);

}  // namespace atlg
