// tf32.cuh -- 3xTF32 tensor-core FP32 GEMM update used by the mixed-precision factorization.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace atlg {

// Pack A (M x K, column-major) / B (K x N, column-major) into the K-major,
// hi/lo-split layouts the tensor-core kernel reads.
void dev_sgemm_tf32x3_pack_a(int M, int K, const float *A, int lda, float *Ap, cudaStream_t st);
void dev_sgemm_tf32x3_pack_b(int K, int N, const float *B, int ldb, float *Bp, cudaStream_t st);
void dev_sgemm_tf32x3_pack_b_rows(int K, int N, const float *B, int ldb, float *Bp, cudaStream_t st);
size_t tf32x3_packed_floats(int rows, int K, bool b_operand);
// C[M x N] += alpha * A * B from the packings (B columns boff .. boff+N-1 of
// a packing made for b_rows_total columns).
void dev_sgemm_tf32x3_packed(int M, int N, int K, float alpha, const float *Ap, const float *Bp, int b_rows_total,
                             int boff, float *C, int ldc, cudaStream_t st);
unsigned tf32_status_read_and_clear();

}  // namespace atlg
