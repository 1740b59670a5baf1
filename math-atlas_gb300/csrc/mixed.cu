// mixed.cu -- mixed-precision dgesv: factor in FP32, recover FP64 accuracy by
// iterative refinement with FP64 residuals; fall back to the FP64 LU when
// refinement does not converge.
//
// No reference counterpart: ATLAS has no mixed-precision solver.  The method
// is iterative refinement as published by Langou, Luszczek, Kurzak, Buttari
// and Dongarra ("Exploiting the performance of 32 bit floating point
// arithmetic in obtaining 64 bit accuracy", SC'06) and used by LAPACK's
// dsgesv; the stopping test is that of dsgesv:
//   ||r_j||_inf <= ||x_j||_inf * ||A||_inf * eps * sqrt(n)   for every column j,
// with eps = 2^-53, at most 30 refinement steps; refinement also stops as
// stalled when the residual fails to halve twice in a row.
//
// GB300 mapping: the FP32 LU is lu.cu's factorization with its trailing
// updates on tcgen05 tensor cores in 3xTF32 (tf32.cu), and the FP32 solves
// are its sgetrs; the FP64 residual r = b - A x is one DGEMM (or
// DGEMV for one right-hand side) on the unmodified FP64 A; conversions and
// norms are elementwise kernels.  All FP64 work on the GPU is the residual,
// the update x += d and the norms; the O(n^3) work is FP32.
#include <float.h>
#include <math.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "lu.cuh"
#include "lu_split.cuh"
#include "mixed.cuh"
#include "trsm.cuh"

namespace atlg {

__global__ void d2s_kernel(int M, int N, const double *__restrict__ A, int lda, float *__restrict__ S, int lds,
                           int *overflow) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)M * N; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % M), j = (int)(e / M);
    const double v = A[i + (size_t)j * lda];
    if (fabs(v) > (double)FLT_MAX) *overflow = 1;
    S[i + (size_t)j * lds] = (float)v;
  }
}
__global__ void s2d_kernel(int M, int N, const float *__restrict__ S, int lds, double *__restrict__ A, int lda) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)M * N; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % M), j = (int)(e / M);
    A[i + (size_t)j * lda] = (double)S[i + (size_t)j * lds];
  }
}
__global__ void axpy_s2d_kernel(int M, int N, const float *__restrict__ S, int lds, double *__restrict__ X, int ldx) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)M * N; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % M), j = (int)(e / M);
    X[i + (size_t)j * ldx] += (double)S[i + (size_t)j * lds];
  }
}
__global__ void copy_d_kernel(int M, int N, const double *__restrict__ S, int lds, double *__restrict__ D, int ldd) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)M * N; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % M), j = (int)(e / M);
    D[i + (size_t)j * ldd] = S[i + (size_t)j * lds];
  }
}

// column-wise max |v| of an M x N block: out[j] (one CTA per column)
template <typename T>
__global__ void __launch_bounds__(256) colmax_kernel(int M, const T *__restrict__ V, int ldv, double *out) {
  __shared__ double sh[8];
  const T *v = V + (size_t)blockIdx.x * ldv;
  double m = 0.0;
  for (int i = threadIdx.x; i < M; i += 256) {
    const double a = fabs((double)v[i]);
    m = a > m ? a : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int q = 0; q < 8; ++q) r = sh[q] > r ? sh[q] : r;
    out[blockIdx.x] = r;
  }
}

// FP64 -> FP32 with IEEE round to nearest even, on the integer pipes: GB300
// retires about two FP64 operations (conversions and compares included) per
// SM per cycle, which would bound a 16384^2 copy at 0.43 ms per operation
// per element.  NaN gives a quiet NaN, magnitudes beyond the float range
// infinity, results below half the smallest float subnormal zero (with the
// sign kept).  value = 1.M * 2^e; for a float subnormal result it is
// F * 2^(e + 97) units of 2^-149, F = 2^52 + M.
__device__ __forceinline__ uint32_t d2f_bits(uint64_t x) {
  const uint32_t sign = (uint32_t)(x >> 32) & 0x80000000u;
  const int E = (int)((x >> 52) & 0x7FF);
  const uint64_t M = x & 0xFFFFFFFFFFFFFull;
  if (E == 0x7FF) return sign | 0x7F800000u | (M ? 0x400000u | (uint32_t)(M >> 29) : 0u);
  const int e = E - 1023;
  if (e > 127) return sign | 0x7F800000u;
  if (e >= -126) {
    uint32_t b = ((uint32_t)(e + 127) << 23) | (uint32_t)(M >> 29);
    const uint32_t rem = (uint32_t)(M & 0x1FFFFFFFu);
    if (rem > 0x10000000u || (rem == 0x10000000u && (b & 1u))) b += 1u;   // a carry may reach infinity
    return sign | b;
  }
  const int sh = -(e + 97);   // 30 .. 53 for the float subnormal range
  if (E == 0 || sh >= 54) return sign;
  const uint64_t F = M | (1ull << 52);
  uint32_t q = (uint32_t)(F >> sh);
  const uint64_t rem = F & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (q & 1u))) q += 1u;
  return sign | q;
}

// The FP32 copy of A and the row sums of |A| (for ||A||_inf) in one pass over
// A: a CTA converts a 256-row x 128-column tile (a thread per row, 16
// columns' loads in flight at a time) and writes its rows' partial sums,
// part[tile column][row]; rowsum_kernel adds the partials in a fixed order.
// The sum of a group of 16 |a| is taken in FP32 from the converted values
// (relative error below 2^-19, enough for a norm used in a stopping test and
// an error estimate) and added in FP64; a group whose FP32 sum could
// overflow (or holds a NaN) is summed again in FP64 from the FP64 values.
// *overflow is set when some |a| exceeds FLT_MAX.
constexpr int kCvRows = 256, kCvCols = 128;

__global__ void __launch_bounds__(kCvRows)
    d2s_rowabs_kernel(int M, int N, const double *__restrict__ A, int lda, float *__restrict__ S, int lds,
                      double *__restrict__ part, int *overflow) {
  const int i = blockIdx.x * kCvRows + threadIdx.x;
  const int j0 = blockIdx.y * kCvCols;
  const int jn = (N - j0 < kCvCols) ? N - j0 : kCvCols;
  if (i >= M) return;
  const unsigned long long *a = reinterpret_cast<const unsigned long long *>(A) + i + (size_t)j0 * lda;
  float *s = S + i + (size_t)j0 * lds;
  double acc = 0.0;
  bool ovf = false;
  for (int g = 0; g < jn; g += 16) {
    unsigned long long v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = (g + q < jn) ? a[(size_t)(g + q) * lda] : 0ull;
    float sum = 0.f;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const uint32_t fb = d2f_bits(v[q]);
      const unsigned long long ax = v[q] & 0x7FFFFFFFFFFFFFFFull;
      ovf |= ax > 0x47EFFFFFE0000000ull && ax <= 0x7FF0000000000000ull;   // FLT_MAX < |a| <= inf
      sum += __uint_as_float(fb & 0x7FFFFFFFu);
      if (g + q < jn) s[(size_t)(g + q) * lds] = __uint_as_float(fb);
    }
    if (sum < 1e37f) {
      acc += (double)sum;
    } else {
      double d = 0.0;
      for (int q = 0; q < 16; ++q) d += fabs(__longlong_as_double((long long)v[q]));
      acc += d;
    }
  }
  if (part) part[(size_t)blockIdx.y * M + i] = acc;
  if (ovf) *overflow = 1;
}

__global__ void rowsum_kernel(int M, int T, const double *__restrict__ part, double *__restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  double s = 0.0;
  for (int t = 0; t < T; ++t) s += part[(size_t)t * M + i];
  rows[i] = s;
}

static int grid_for(long work) {
  long b = (work + 255) / 256;
  if (b > 16L * 152) b = 16L * 152;
  if (b < 1) b = 1;
  return (int)b;
}

static std::vector<double> colmax_host(int M, int N, const double *V, int ldv, double *dtmp, cudaStream_t st) {
  colmax_kernel<double><<<N, 256, 0, st>>>(M, V, ldv, dtmp);
  note_launch();
  std::vector<double> h(N);
  ATLG_CHECK(cudaMemcpyAsync(h.data(), dtmp, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  return h;
}

static bool g_refine_chained = true;
void set_refine_trsv_chained(bool on) { g_refine_chained = on; }

// column maxima of two M x N blocks with one host synchronisation:
// v[j] = max_i |V(i,j)|, w[j] = max_i |W(i,j)| (dtmp holds 2N doubles)
static void colmax2_host(int M, int N, const double *V, int ldv, const double *W, int ldw, double *dtmp,
                         std::vector<double> &v, std::vector<double> &w, cudaStream_t st) {
  colmax_kernel<double><<<N, 256, 0, st>>>(M, V, ldv, dtmp);
  colmax_kernel<double><<<N, 256, 0, st>>>(M, W, ldw, dtmp + N);
  note_launch(2);
  std::vector<double> h(2 * (size_t)N);
  ATLG_CHECK(cudaMemcpyAsync(h.data(), dtmp, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  v.assign(h.begin(), h.begin() + N);
  w.assign(h.begin() + N, h.end());
}

int dev_dgesv_mixed(int n, int nrhs, double *A, int lda, int *ipiv, const double *B, int ldb, double *X, int ldx,
                    MixedResult *res, cudaStream_t st) {
  Context &c = ctx();
  res->iters = 0;
  res->status = 0;
  res->berr.assign(nrhs, 0.0);
  res->ferr.assign(nrhs, 0.0);
  if (n == 0 || nrhs == 0) return 0;
  const int lds = (n + 3) & ~3;               // 16-byte aligned FP32 columns (TMA)
  float *S = static_cast<float *>(c.buffer(kBufW1, sizeof(float) * (size_t)lds * n));
  const int ldr = (n + 1) & ~1;
  double *R = static_cast<double *>(c.buffer(kBufW2, sizeof(double) * (size_t)ldr * nrhs));
  float *R32 = static_cast<float *>(c.buffer(kBufW5, sizeof(float) * (size_t)lds * nrhs + 4096));
  double *small = static_cast<double *>(c.buffer(kBufInfo, sizeof(double) * (size_t)(2 * n + 2 * nrhs + 16)));
  int *dinfo = reinterpret_cast<int *>(small);
  int *dovf = dinfo + 1;
  double *dtmp = small + 2;
  double *drows = dtmp + nrhs + 1;

  // The FP32 copy of A with the row sums of |A| in the same pass, ||A||_inf
  // and ||b_j||_inf, then the FP32 factorization; info, the overflow flag and
  // the norms come back with one host synchronisation after it.
  ATLG_CHECK(cudaMemsetAsync(dinfo, 0, 2 * sizeof(int), st));
  {
    const int tiles = (n + kCvCols - 1) / kCvCols;
    double *part = static_cast<double *>(c.buffer(kBufRowPart, sizeof(double) * (size_t)tiles * n));
    d2s_rowabs_kernel<<<dim3((n + kCvRows - 1) / kCvRows, tiles), kCvRows, 0, st>>>(n, n, A, lda, S, lds, part,
                                                                                   dovf);
    rowsum_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, tiles, part, drows);
    colmax_kernel<double><<<1, 256, 0, st>>>(n, drows, n, dtmp);
    colmax_kernel<double><<<nrhs, 256, 0, st>>>(n, B, ldb, dtmp + 1);
    note_launch(4);
    ATLG_CHECK(cudaGetLastError());
  }
  dev_sgetrf_tc(n, n, S, lds, ipiv, dinfo, st);
  std::vector<double> head(3 + (size_t)nrhs);
  ATLG_CHECK(cudaMemcpyAsync(head.data(), small, sizeof(double) * head.size(), cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  int hinfo[2];
  memcpy(hinfo, head.data(), sizeof(hinfo));
  const double anrm = head[2];
  std::vector<double> bnrm(head.begin() + 3, head.end());
  const double eps = ldexp(1.0, -53);
  const double cte = anrm * eps * sqrt((double)n);
  bool fallback = hinfo[0] != 0 || hinfo[1] != 0;

  int iter = 0;
  if (!fallback) {
    // one right-hand side: the row permutation is computed once and every
    // solve is a gather plus two single-launch triangular solves
    // (a gather plus two chained triangular solves whose 128 x 128 block
    // inverses and couplings are formed once here)
    int *perm = nullptr;
    float *tmp32 = nullptr, *wsL = nullptr, *wsU = nullptr;
    const bool chained = g_refine_chained;
    if (nrhs == 1) {
      perm = static_cast<int *>(c.buffer(kBufV1, sizeof(int) * (size_t)n + sizeof(float) * (size_t)n + 256));
      tmp32 = reinterpret_cast<float *>(perm + ((n + 63) & ~63));
      dev_perm_from_ipiv(ipiv, n, perm, st);
      if (chained) {
        wsL = static_cast<float *>(c.buffer(kBufTrsvL, sizeof(float) * strsv_chain_ws_floats(n)));
        wsU = static_cast<float *>(c.buffer(kBufTrsvU, sizeof(float) * strsv_chain_ws_floats(n)));
        dev_strsv_chain_prepare(kLower, kUnit, n, S, lds, wsL, st);
        dev_strsv_chain_prepare(kUpper, kNonUnit, n, S, lds, wsU, st);
      }
    }
    auto solve32 = [&](float *v) {
      if (nrhs == 1 && chained) dev_sgetrs_perm_chain(n, S, lds, perm, v, tmp32, wsL, wsU, st);
      else if (nrhs == 1) dev_sgetrs_perm(n, S, lds, perm, v, tmp32, st);
      else dev_sgetrs(kColMajor, kNoTrans, n, nrhs, S, lds, ipiv, v, lds, st);
    };
    // x0 = (A32)^-1 b in FP32, promoted
    d2s_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, B, ldb, R32, lds, dovf);
    note_launch();
    solve32(R32);
    s2d_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, R32, lds, X, ldx);
    note_launch();
    double prev = INFINITY;
    int slow = 0;
    const int kItMax = 30;
    bool conv = false;
    for (iter = 0; iter <= kItMax; ++iter) {
      // r = b - A x  (FP64)
      copy_d_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, B, ldb, R, ldr);
      note_launch();
      dev_dgemm(kNoTrans, kNoTrans, n, nrhs, n, -1.0, A, lda, X, ldx, 1.0, R, ldr, st);
      std::vector<double> rn, xn;
      colmax2_host(n, nrhs, R, ldr, X, ldx, dtmp, rn, xn, st);   // (dtmp spans the row sums, used only above)
      conv = true;
      double rmax = 0.0;
      for (int j = 0; j < nrhs; ++j) {
        if (!(rn[j] <= xn[j] * cte)) conv = false;
        rmax = rn[j] > rmax ? rn[j] : rmax;
        const double den = anrm * xn[j] + bnrm[j];
        res->berr[j] = den > 0 ? rn[j] / den : 0.0;
      }
      if (conv || iter == kItMax) break;
      if (!(rmax < 0.5 * prev)) {
        if (++slow >= 2) break;   // stalled
      } else {
        slow = 0;
      }
      prev = rmax;
      // d = (A32)^-1 r in FP32; x += d
      d2s_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, R, ldr, R32, lds, dovf);
      note_launch();
      solve32(R32);
      axpy_s2d_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, R32, lds, X, ldx);
      note_launch();
    }
    if (iter > 0) {
      // forward-error estimate ||d||/||x|| from the last FP32 correction (R32
      // still holds it: the loop ends on a residual, before another solve)
      s2d_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, R32, lds, R, ldr);
      note_launch();
      std::vector<double> d2, x2;
      colmax2_host(n, nrhs, R, ldr, X, ldx, dtmp, d2, x2, st);
      for (int j = 0; j < nrhs; ++j) res->ferr[j] = x2[j] > 0 ? d2[j] / x2[j] : 0.0;
    }
    res->iters = iter;
    fallback = !conv;
  }
  if (fallback) {
    // FP64 LU of a copy of A and the FP64 solve; the normwise backward error
    // is measured against the untouched A, then the factors are returned in A
    // (LAPACK dsgesv convention for the fallback).
    res->status = 1;
    const int ldf = (n + 1) & ~1;
    double *F = static_cast<double *>(c.buffer(kBufW6, sizeof(double) * (size_t)ldf * n));
    copy_d_kernel<<<grid_for((long)n * n), 256, 0, st>>>(n, n, A, lda, F, ldf);
    note_launch();
    // FP64-accurate LU with its O(n^3) updates on the tensor pipe (lu_split.cu)
    const int i64 = dev_dgetrf_split(n, F, ldf, ipiv, 8, 1024, st);
    if (i64 != 0) {
      res->status = 2;
      copy_d_kernel<<<grid_for((long)n * n), 256, 0, st>>>(n, n, F, ldf, A, lda);
      note_launch();
      ATLG_CHECK(cudaStreamSynchronize(st));
      return i64;
    }
    copy_d_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, B, ldb, X, ldx);
    note_launch();
    dev_dgetrs(kColMajor, kNoTrans, n, nrhs, F, ldf, ipiv, X, ldx, st);
    copy_d_kernel<<<grid_for((long)n * nrhs), 256, 0, st>>>(n, nrhs, B, ldb, R, ldr);
    note_launch();
    dev_dgemm(kNoTrans, kNoTrans, n, nrhs, n, -1.0, A, lda, X, ldx, 1.0, R, ldr, st);
    std::vector<double> rn = colmax_host(n, nrhs, R, ldr, dtmp, st);
    std::vector<double> xn = colmax_host(n, nrhs, X, ldx, dtmp, st);
    for (int j = 0; j < nrhs; ++j) {
      const double den = anrm * xn[j] + bnrm[j];
      res->berr[j] = den > 0 ? rn[j] / den : 0.0;
      res->ferr[j] = 0.0;
    }
    copy_d_kernel<<<grid_for((long)n * n), 256, 0, st>>>(n, n, F, ldf, A, lda);
    note_launch();
    ATLG_CHECK(cudaStreamSynchronize(st));
  }
  return 0;
}

// SA = A in FP32 (LAPACK dlag2s, the conversion dsgesv makes): returns 1
// when some |a| exceeds FLT_MAX (those entries become infinities), else 0.
int dev_dlag2s(int M, int N, const double *A, int lda, float *SA, int ldsa, cudaStream_t st) {
  if (M <= 0 || N <= 0) return 0;
  Context &c = ctx();
  int *flag = static_cast<int *>(c.buffer(kBufFlag, sizeof(int)));
  ATLG_CHECK(cudaMemsetAsync(flag, 0, sizeof(int), st));
  d2s_rowabs_kernel<<<dim3((M + kCvRows - 1) / kCvRows, (N + kCvCols - 1) / kCvCols), kCvRows, 0, st>>>(
      M, N, A, lda, SA, ldsa, nullptr, flag);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
  int h = 0;
  ATLG_CHECK(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  ATLG_CHECK(cudaStreamSynchronize(st));
  return h;
}

}  // namespace atlg
