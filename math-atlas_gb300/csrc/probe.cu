// probe.cu -- arithmetic-pipe throughput probes used as roofline
// denominators where the measured peaks have no entry (FP64 and FP32
// on the CUDA cores, FP64 on the tensor cores): every thread runs 16
// independent FMA chains (every warp 4 independent FP64 mma.sync chains) for
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

// FP64 tensor-core probe: mma.sync with f64 operands and accumulators, the
// only FP64 tensor-core instruction form sm_103a has (tcgen05 has no f64
// kind).  Shapes: 0 = m8n8k4 (512 flops per warp instruction), 1 = m16n8k4
// (1024), 2 = m16n8k16 (4096).  Four independent accumulator chains per warp.
template <int SHAPE>
__global__ void __launch_bounds__(256) dmma_probe_kernel(double *out, int iters, double a, double b) {
  double c[4][4];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int i = 0; i < 4; ++i) c[q][i] = 1e-3 * (threadIdx.x + i + q);
  double av[8], bv[4];
#pragma unroll
  for (int i = 0; i < 8; ++i) av[i] = a + 1e-9 * i;
#pragma unroll
  for (int i = 0; i < 4; ++i) bv[i] = b + 1e-9 * i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (SHAPE == 0) {
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                     : "+d"(c[q][0]), "+d"(c[q][1])
                     : "d"(av[0]), "d"(bv[0]));
      } else if (SHAPE == 1) {
        asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
                     "{%0,%1,%2,%3};\n"
                     : "+d"(c[q][0]), "+d"(c[q][1]), "+d"(c[q][2]), "+d"(c[q][3])
                     : "d"(av[0]), "d"(av[1]), "d"(bv[0]));
      } else {
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                     "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
                     : "+d"(c[q][0]), "+d"(c[q][1]), "+d"(c[q][2]), "+d"(c[q][3])
                     : "d"(av[0]), "d"(av[1]), "d"(av[2]), "d"(av[3]), "d"(av[4]), "d"(av[5]), "d"(av[6]),
                       "d"(av[7]), "d"(bv[0]), "d"(bv[1]), "d"(bv[2]), "d"(bv[3]));
      }
    }
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int i = 0; i < 4; ++i) s += c[q][i];
  if (s == -12345.25) out[blockIdx.x] = s;   // keeps the chains live; never taken for these inputs
}

template <int SHAPE>
static double dmma_probe(int iters) {
  Context &c = ctx();
  double *out = static_cast<double *>(c.buffer(kBufW5, sizeof(double) * 4096));
  const int blocks = c.num_sms * 8, threads = 256;
  cudaEvent_t e0 = c.event(), e1 = c.event();
  dmma_probe_kernel<SHAPE><<<blocks, threads, 0, c.stream>>>(out, 8, 1e-3, 1e-3);   // warm-up
  ATLG_CHECK(cudaEventRecord(e0, c.stream));
  dmma_probe_kernel<SHAPE><<<blocks, threads, 0, c.stream>>>(out, iters, 1e-3, 1e-3);
  ATLG_CHECK(cudaEventRecord(e1, c.stream));
  ATLG_CHECK(cudaEventSynchronize(e1));
  ATLG_CHECK(cudaGetLastError());
  float ms = 0.f;
  ATLG_CHECK(cudaEventElapsedTime(&ms, e0, e1));
  c.pool.push_back(e0);
  c.pool.push_back(e1);
  const double flops_per_mma = SHAPE == 0 ? 512.0 : SHAPE == 1 ? 1024.0 : 4096.0;
  const double warps = (double)blocks * threads / 32.0;
  return flops_per_mma * 4.0 * iters * warps / (ms * 1e-3) / 1e12;
}

double probe_fp64_tflops() { return probe<double>(4000); }
void probe_fp64_mma_tflops(double *m8n8k4, double *m16n8k4, double *m16n8k16) {
  if (m8n8k4) *m8n8k4 = dmma_probe<0>(1000);
  if (m16n8k4) *m16n8k4 = dmma_probe<1>(500);
  if (m16n8k16) *m16n8k16 = dmma_probe<2>(125);
}
double probe_fp32_tflops() { return probe<float>(40000); }

}  // namespace atlg
