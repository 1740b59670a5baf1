// probe.cu -- arithmetic-pipe throughput probes used as roofline
// denominators where the measured peaks have no entry (FP64 and FP32
// on the CUDA cores): every thread runs 16 independent FMA chains for
// `iters` rounds, the grid fills every SM, and the kernel is timed with CUDA
// events on the library stream.
#include "common.cuh"
#include "context.cuh"

namespace atlg {

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T *out, int iters, T a, T b) {
  T r[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) r[i] = T(threadIdx.x) * T(1e-3) + T(i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 16; ++i) r[i] = fma(r[i], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int i = 0; i < 16; ++i) s += r[i];
  if (s == T(-12345.25)) out[blockIdx.x] = s;   // keeps the chains live; never taken for these inputs
}

template <typename T>
static double probe(int iters) {
  Context &c = ctx();
  T *out = static_cast<T *>(c.buffer(kBufW5, sizeof(T) * 4096));
  const int blocks = c.num_sms * 8, threads = 256;
  cudaEvent_t e0 = c.event(), e1 = c.event();
  fma_probe_kernel<T><<<blocks, threads, 0, c.stream>>>(out, 16, T(1.0000001), T(1e-9));   // warm-up
  ATLG_CHECK(cudaEventRecord(e0, c.stream));
  fma_probe_kernel<T><<<blocks, threads, 0, c.stream>>>(out, iters, T(1.0000001), T(1e-9));
  ATLG_CHECK(cudaEventRecord(e1, c.stream));
  ATLG_CHECK(cudaEventSynchronize(e1));
  float ms = 0.f;
  ATLG_CHECK(cudaEventElapsedTime(&ms, e0, e1));
  c.pool.push_back(e0);
  c.pool.push_back(e1);
  return 2.0 * 16.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
}

double probe_fp64_tflops() { return probe<double>(4000); }
double probe_fp32_tflops() { return probe<float>(40000); }

}  // namespace atlg
