// iamax.cu -- cblas_idamax / cblas_isamax on GB300: the index of the first
// element of largest magnitude, with the reference's exact semantics.
//
// Reference: cblas_i?amax (AtlasBase/Clint/cblas-lvl1.base:408-420) returns
// ATL_i?amax(N, X, incX) when N > 0 and incX > 0, else 0; ATL_i?amax
// (AtlasBase/Clint/atlas-lvl1.base:1148-1340) scans X in order keeping a pair
// (P, Q), initially (0, 0), and for each x
//     if (x <= P && x >= Q)  nothing
//     else if (x > P)        (P, Q) = (x, -x), remember x's index
//     else                   (P, Q) = (-x, x), remember x's index
// and returns the last remembered index (0 when N < 2 or when nothing was
// remembered); the unit-stride form also returns 0 when it ends with P == 0
// or Q == 0.  Without NaNs this is the first index of max |x|.  A NaN fails
// every comparison, so it is always remembered and leaves (P, Q) = (NaN, NaN);
// the next element is then always remembered and gives (|x|, -|x|) when
// x <= 0 but the inverted pair (-x, x) when x > 0, after which elements keep
// being remembered until the pair is ordered (P >= Q) again.
//
// GB300 design (HBM-bound, 8 bytes per element read once): one launch.  Each
// CTA reduces a contiguous chunk to (largest |x| key, first index, last NaN
// index) on integer keys (the bit pattern of |x| orders as |x| for non-NaN x),
// writes that record, and the last CTA to finish merges the records.  Without
// a NaN the answer is the merged first maximum.  With one, its thread 0 runs
// the reference's comparisons from the last NaN on until the pair is ordered
// again (position r, value m), and the CTA finishes with the first maximum
// after r: a scan of the rest of r's chunk plus the later chunks' records.
#include <stdint.h>

#include "common.cuh"
#include "context.cuh"
#include "iamax.cuh"

namespace atlg {

constexpr int kIaThreads = 256;
constexpr int kIaUnroll = 8;

__device__ unsigned g_iamax_done;   // CTAs finished in the current call; the merging CTA resets it

struct IamaxRec {
  unsigned long long key;   // |x| bits of the chunk's first maximum (0 when none)
  long long idx;            // its index, -1 when none
  long long nan;            // last NaN index in the chunk, -1 when none
};

template <typename T> struct IaKey;
template <> struct IaKey<double> {
  __device__ static unsigned long long key(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  }
  static constexpr unsigned long long kInf = 0x7ff0000000000000ull;
};
template <> struct IaKey<float> {
  __device__ static unsigned long long key(float x) { return (unsigned)__float_as_uint(x) & 0x7fffffffu; }
  static constexpr unsigned long long kInf = 0x7f800000ull;
};

// (key, idx) order: larger key first, then smaller index
__device__ __forceinline__ bool ia_better(unsigned long long k1, long long i1, unsigned long long k2, long long i2) {
  return k1 > k2 || (k1 == k2 && i1 >= 0 && (i2 < 0 || i1 < i2));
}

// Block reduction of (key, idx, nan) to thread 0's values.
__device__ void ia_block_reduce(unsigned long long &key, long long &idx, long long &nan) {
  __shared__ unsigned long long sk[kIaThreads / 32];
  __shared__ long long si[kIaThreads / 32], sn[kIaThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long k2 = __shfl_down_sync(0xffffffffu, key, o);
    const long long i2 = __shfl_down_sync(0xffffffffu, idx, o);
    const long long n2 = __shfl_down_sync(0xffffffffu, nan, o);
    if (ia_better(k2, i2, key, idx)) { key = k2; idx = i2; }
    nan = n2 > nan ? n2 : nan;
  }
  __syncthreads();
  if (lane == 0) { sk[w] = key; si[w] = idx; sn[w] = nan; }
  __syncthreads();
  if (w == 0) {
    key = lane < kIaThreads / 32 ? sk[lane] : 0ull;
    idx = lane < kIaThreads / 32 ? si[lane] : -1;
    nan = lane < kIaThreads / 32 ? sn[lane] : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_down_sync(0xffffffffu, key, o);
      const long long i2 = __shfl_down_sync(0xffffffffu, idx, o);
      const long long n2 = __shfl_down_sync(0xffffffffu, nan, o);
      if (ia_better(k2, i2, key, idx)) { key = k2; idx = i2; }
      nan = n2 > nan ? n2 : nan;
    }
  }
}

template <typename T> struct IaVec;
template <> struct IaVec<double> { using type = double2; };
template <> struct IaVec<float> { using type = float4; };

// First maximum and last NaN over elements [b, e) of X (stride inc), this
// CTA's threads, coalesced for inc = 1.  Every thread visits its elements in
// increasing index order, so `k > key` keeps a thread's first maximum and
// `nan = i` its last NaN.  Unit stride from a 16-byte aligned start reads
// 16-byte vectors (kIaUnroll of them in flight per thread), the rest one
// element at a time.
template <typename T>
__device__ void ia_scan(const T *__restrict__ X, long long inc, long long b, long long e, unsigned long long &key,
                        long long &idx, long long &nan) {
  auto visit = [&](T x, long long i) {
    const unsigned long long k = IaKey<T>::key(x);
    if (k > IaKey<T>::kInf) nan = i;
    else if (k > key) { key = k; idx = i; }
  };
  if (inc == 1 && (reinterpret_cast<uintptr_t>(X + b) & 15) == 0) {
    using V = typename IaVec<T>::type;
    constexpr int VE = 16 / (int)sizeof(T);
    const long long nv = (e - b) / VE;
    const V *xv = reinterpret_cast<const V *>(X + b);
    for (long long q0 = threadIdx.x; q0 < nv; q0 += (long long)kIaUnroll * kIaThreads) {
      V v[kIaUnroll];
#pragma unroll
      for (int u = 0; u < kIaUnroll; ++u) {
        const long long q = q0 + (long long)u * kIaThreads;
        if (q < nv) v[u] = xv[q];
      }
#pragma unroll
      for (int u = 0; u < kIaUnroll; ++u) {
        const long long q = q0 + (long long)u * kIaThreads;
        if (q < nv) {
          const T *ve = reinterpret_cast<const T *>(&v[u]);
#pragma unroll
          for (int t = 0; t < VE; ++t) visit(ve[t], b + q * VE + t);
        }
      }
    }
    for (long long i = b + nv * VE + threadIdx.x; i < e; i += kIaThreads) visit(X[i], i);
    return;
  }
  for (long long i0 = b + threadIdx.x; i0 < e; i0 += (long long)kIaUnroll * kIaThreads) {
    T v[kIaUnroll];
#pragma unroll
    for (int u = 0; u < kIaUnroll; ++u) {
      const long long i = i0 + (long long)u * kIaThreads;
      v[u] = i < e ? X[i * inc] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kIaUnroll; ++u) {
      const long long i = i0 + (long long)u * kIaThreads;
      if (i < e) {
        const unsigned long long k = IaKey<T>::key(v[u]);
        if (k > IaKey<T>::kInf) nan = i;            // indexes rise within a thread
        else if (k > key) { key = k; idx = i; }
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kIaThreads, 4)
    iamax_kernel(long long n, const T *__restrict__ X, long long inc, int unit, long long chunk, IamaxRec *rec,
                 int *result) {
  __shared__ int s_last;
  __shared__ long long s_r;
  __shared__ T s_m;
  unsigned long long key = 0;
  long long idx = -1, nan = -1;
  const long long b = (long long)blockIdx.x * chunk;
  const long long e = (b + chunk < n) ? b + chunk : n;
  ia_scan<T>(X, inc, b, e, key, idx, nan);
  ia_block_reduce(key, idx, nan);
  if (threadIdx.x == 0) {
    rec[blockIdx.x] = IamaxRec{key, idx, nan};
    __threadfence();
    const unsigned done = atomicAdd(&g_iamax_done, 1u);
    s_last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  // ---- the last CTA merges
  __threadfence();
  const int nrec = gridDim.x;
  key = 0; idx = -1; nan = -1;
  for (int t = threadIdx.x; t < nrec; t += kIaThreads) {   // L2 reads: written by other CTAs
    const unsigned long long rk = __ldcg(&rec[t].key);
    const long long ri = __ldcg(&rec[t].idx), rn = __ldcg(&rec[t].nan);
    if (ia_better(rk, ri, key, idx)) { key = rk; idx = ri; }
    nan = rn > nan ? rn : nan;
  }
  ia_block_reduce(key, idx, nan);
  __shared__ unsigned long long s_key;
  __shared__ long long s_idx, s_nan;
  if (threadIdx.x == 0) { s_key = key; s_idx = idx; s_nan = nan; }
  __syncthreads();
  if (s_nan < 0) {   // no NaN: the first maximum, 0 when every |x| is 0
    if (threadIdx.x == 0) {
      *result = (s_key == 0 || s_idx < 0) ? 0 : (int)s_idx;
      g_iamax_done = 0;
    }
    return;
  }
  // NaN: the reference's comparisons from the last NaN until (P, Q) is ordered
  if (threadIdx.x == 0) {
    T P = X[s_nan * inc], Q = P;   // both NaN
    long long j = s_nan + 1, r = -1;
    for (; j < n; ++j) {
      const T x = X[j * inc];
      if (x <= P && x >= Q) continue;        // cannot hold while P, Q are NaN or inverted
      if (x > P) { P = x; Q = -x; }
      else { P = -x; Q = x; }
      if (P >= Q) { r = j; break; }
    }
    s_r = r;
    s_m = P;
  }
  __syncthreads();
  const long long r = s_r;
  if (r < 0) {       // never ordered again: every element after the NaN was remembered
    if (threadIdx.x == 0) { *result = (int)(n - 1); g_iamax_done = 0; }
    return;
  }
  // first maximum after r: the rest of r's chunk, then the later records
  const long long cr = r / chunk;
  const long long ce = ((cr + 1) * chunk < n) ? (cr + 1) * chunk : n;
  key = 0; idx = -1; nan = -1;
  ia_scan<T>(X, inc, r + 1, ce, key, idx, nan);
  for (long long t = cr + 1 + threadIdx.x; t < nrec; t += kIaThreads) {
    const unsigned long long rk = __ldcg(&rec[t].key);
    const long long ri = __ldcg(&rec[t].idx);
    if (ia_better(rk, ri, key, idx)) { key = rk; idx = ri; }
  }
  ia_block_reduce(key, idx, nan);
  if (threadIdx.x == 0) {
    const T m = s_m;                         // P >= 0 here
    long long res = r;
    bool zero = (m == T(0));
    if (idx >= 0 && key > IaKey<T>::key(m)) { res = idx; zero = false; }
    *result = (unit && zero) ? 0 : (int)res;
    g_iamax_done = 0;
  }
}

template <typename T>
static void iamax_impl(int N, const T *X, int incX, int unit, int *result, cudaStream_t st) {
  Context &c = ctx();
  long long per = (long long)kIaThreads * kIaUnroll * 2;
  long long grid = ((long long)N + per - 1) / per;
  const long long cap = 4LL * c.num_sms;   // one wave at 4 CTAs per SM
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  // chunks of a multiple of 8 elements keep every chunk's start 16-byte
  // aligned when X is (the vector path of ia_scan)
  const long long chunk = (((long long)N + grid - 1) / grid + 7) / 8 * 8;
  grid = ((long long)N + chunk - 1) / chunk;
  IamaxRec *rec = static_cast<IamaxRec *>(c.buffer(kBufIamax, sizeof(IamaxRec) * (size_t)grid));
  iamax_kernel<T><<<(int)grid, kIaThreads, 0, st>>>(N, X, incX, unit, chunk, rec, result);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

// N >= 2, incX >= 1; `unit` selects the unit-stride form's final P == 0 check.
void dev_idamax(int N, const double *X, int incX, int unit, int *result, cudaStream_t st) {
  iamax_impl<double>(N, X, incX, unit, result, st);
}
void dev_isamax(int N, const float *X, int incX, int unit, int *result, cudaStream_t st) {
  iamax_impl<float>(N, X, incX, unit, result, st);
}

}  // namespace atlg
