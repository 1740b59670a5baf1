// iamax.cuh -- device-pointer index of the first element of largest magnitude.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// ATL_i?amax semantics for N >= 2, incX >= 1 (device X, device int result,
// 0-based).  unit = 1 applies the unit-stride form's final check (0 when the
// scan ends with a zero magnitude), unit = 0 the strided form's.
void dev_idamax(int N, const double *X, int incX, int unit, int *result, cudaStream_t st);
void dev_isamax(int N, const float *X, int incX, int unit, int *result, cudaStream_t st);

}  // namespace atlg
