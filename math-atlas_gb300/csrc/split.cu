// split.cu -- split-precision DGEMM: C = alpha*op(A)*op(B) + beta*C in FP64
// computed from 7-bit integer slices of A and B on the fifth-generation
// tensor cores (tcgen05, kind::f16), accumulated exactly, recombined in FP64.
//
// No reference counterpart (ATLAS's GEMM is FP64 throughout).  The method is
// the Ozaki scheme of error-free splitting (Ozaki, Ogita, Oishi, Rump,
// Numer. Algorithms 59, 2012) in its integer form (Ootomo, Ozaki, Yokota,
// IJHPCA 2024: "DGEMM on integer matrix multiplication unit"):
//   op(A) = diag(2^ea) sum_t 2^(-7(t+1)) A_t,  op(B) = (sum_u 2^(-7(u+1)) B_u) diag(2^eb)
// with per-row (A) / per-column (B) power-of-two scales and integer digit
// matrices |A_t|, |B_u| <= 127, and
//   op(A) op(B) ~= diag(2^ea) [ sum_{t+u<=s-1} 2^(-7(t+u+2)) A_t B_u ] diag(2^eb).
//
// GB300 mapping.  sm_103a has no tcgen05 INT8 MMA (kind::i8 does not
// assemble), so the digits are stored as FP16 -- every integer of magnitude
// <= 2048 is exact in FP16 -- and multiplied with tcgen05.mma kind::f16 into
// FP32 tensor memory.  A product of two digits is below 2^14; 1024 of them
// sum below 2^24, so an FP32 accumulator over a K chunk of 1024 holds the
// exact integer (the GPU test checks this bit for bit).  After each chunk the
// epilogue warps move the accumulator out of tensor memory (tcgen05.ld),
// convert it to int32 and add it to per-thread int32 sums that collect every
// chunk and every slice pair of one diagonal t+u = d (at most 8 pairs x 16
// chunks x 2^24 < 2^31 for K <= 16384: exact).  Each diagonal is then added
// into C in FP64 with one exact power-of-two scaling, smallest diagonal
// first.  K > 16384 is split into pieces accumulated through beta = 1.
//
// Kernel structure (one 128 x 256 tile of C per CTA, 18 warps):
//   warp 0   TMA producer: 128 x 64 and 256 x 64 FP16 tiles of A_t and B_u
//            (K-major, 128-byte swizzle) into a 4-stage shared-memory ring
//            (48 KB per stage: 512 MMA cycles of 128x256x16 cover the TMA
//            latency);
//   warp 1   allocates all 512 tensor-memory columns (two 256-column FP32
//            accumulators) and issues the MMAs (one thread), committing to
//            the ring's empty barriers and the accumulator-full barriers;
//   warps 2-17 epilogue: warp w reads tensor-memory lane quarter w % 4;
//            each thread owns one row of the tile and 64 of its 256
//            columns (int32 sums).
// Every wait is bounded; a timeout sets the status word and an abort flag
// that every role polls, so the CTA drains, frees its tensor memory and exits.
#include <cuda_fp16.h>
#include <math.h>

#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "split.cuh"
#include "tc.cuh"

namespace atlg {

__device__ unsigned g_split_status;

constexpr int kSliceBits = 7;
constexpr int TM = 128, TN = 256, KB = 64, KCHUNK_BLOCKS = 16;   // 16 x 64 = 1024 = exact FP32 chunk
constexpr int STAGES = 4;
constexpr int STAGE_BYTES = (TM + TN) * KB * 2;                  // 48 KB
constexpr int EPI_WARPS = 16;
constexpr int SPLIT_THREADS = 64 + EPI_WARPS * 32;             // 2 + 16 warps
constexpr int EPI_COLS = 64;                                   // columns per epilogue thread
constexpr int SPLIT_SMEM = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int kRasterN = 8;                                    // column tiles per raster group

// --------------------------------------------------------------- scaling
// |x| as an integer key: the bit pattern of |x| orders exactly as |x| for x
// not NaN; NaN maps to 0, so a maximum over keys ignores NaN as fmax does.
// Integer max/compare keeps the scan off GB300's narrow FP64 pipe.
__device__ __forceinline__ long long abs_bits(double x) {
  const long long b = __double_as_longlong(x) & 0x7fffffffffffffffLL;
  return b > 0x7ff0000000000000LL ? 0LL : b;
}

// ex[r] = exponent e with max_k |In(r,k)| < 2^e (0 for an all-zero vector);
// In(r,k) = In[r*rs + k*ks].  Contiguous-in-k vectors: a warp per vector;
// otherwise 32 consecutive vectors per CTA, 8 warps striding over k.
__global__ void __launch_bounds__(256) vec_exp_kernel(int R, int Kd, const double *__restrict__ In, long rs, long ks,
                                                      int *__restrict__ ex) {
  __shared__ long long part[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long m = 0;
  int r;
  if (ks == 1) {
    r = blockIdx.x * 8 + w;
    if (r < R)
      for (int k = lane; k < Kd; k += 32) m = max(m, abs_bits(In[(size_t)r * rs + k]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if (lane == 0 && r < R) {
      int e = 0;
      if (m > 0) frexp(__longlong_as_double(m), &e);
      ex[r] = e;
    }
  } else {
    r = blockIdx.x * 32 + lane;
    if (r < R)
      for (int k = w; k < Kd; k += 8) m = max(m, abs_bits(In[(size_t)r * rs + (size_t)k * ks]));
    part[w][lane] = m;
    __syncthreads();
    if (w == 0 && r < R) {
      long long mm = 0;
      for (int q = 0; q < 8; ++q) mm = max(mm, part[q][lane]);
      int e = 0;
      if (mm > 0) frexp(__longlong_as_double(mm), &e);
      ex[r] = e;
    }
  }
}

// Digit split of In (R x Kd, strides rs/ks) into s FP16 slices
// Out[(t*Rp + r)*Kp + k], zero outside R x Kd.  With x = In * 2^-e in
// (-1, 1), digit t = trunc(128 * remainder_t): the binary fraction of |x| cut
// into 7-bit groups, with the sign of x.  A finite x is exact in 56 fraction
// bits of fixed point taken straight from its significand and exponent
// (integer shifts, no FP64 arithmetic; the FP64 recurrence
// x *= 128, d = trunc(x), x -= d is exact, so the digits are the same).
// Values the fixed point cannot hold (NaN, infinity, |x| >= 1 in a vector
// whose maximum was not finite) take that FP64 recurrence.
__device__ __forceinline__ void digits_of(double v, int e, int s, __half *h) {
  const long long b = __double_as_longlong(v);
  const int ef = (int)((b >> 52) & 0x7ff);
  const int E = (ef ? ef : 1) - 1075;            // |v| = mant * 2^E
  const int sh = 56 - (e - E);                   // frac56 = mant * 2^sh
  if (ef == 0x7ff || (ef != 0 && sh > 3) || sh > 55) {
    double x = ldexp(v, -e);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      x *= 128.0;
      const double d = trunc(x);
      x -= d;
      if (t < s) h[t] = __double2half((float)d);
    }
    return;
  }
  const unsigned long long mant = (unsigned long long)(b & 0xfffffffffffffLL) | (ef ? (1ull << 52) : 0ull);
  unsigned long long f = 0;
  if (sh >= 0) f = mant << sh;
  else if (sh > -64) f = mant >> (-sh);
  const int sg = (b < 0) ? -1 : 1;
#pragma unroll
  for (int t = 0; t < 8; ++t)
    if (t < s) h[t] = __int2half_rn(sg * (int)((f >> (49 - 7 * t)) & 127ull));
}

__global__ void __launch_bounds__(256) slice_kernel(int R, int Kd, int Rp, int Kp, int s, const double *__restrict__ In,
                                                    long rs, long ks, const int *__restrict__ ex,
                                                    __half *__restrict__ Out) {
  __shared__ double tile[32][33];
  __shared__ int tex[32];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  if (threadIdx.x < 32) tex[threadIdx.x] = (r0 + threadIdx.x < R) ? ex[r0 + threadIdx.x] : 0;
  // load: coalesce along whichever dimension is contiguous
  for (int q = ty; q < 32; q += 8) {
    int r, k;
    if (ks == 1) { r = r0 + q; k = k0 + tx; } else { r = r0 + tx; k = k0 + q; }
    double v = 0.0;
    if (r < R && k < Kd) v = In[(size_t)r * rs + (size_t)k * ks];
    if (ks == 1) tile[q][tx] = v; else tile[tx][q] = v;
  }
  __syncthreads();
  // store: consecutive threads -> consecutive k
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + q, k = k0 + tx;
    if (r >= Rp || k >= Kp) continue;
    __half h[8];
    digits_of(tile[q][tx], tex[q], s, h);
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (t < s) Out[((size_t)t * Rp + r) * Kp + k] = h[t];
  }
}

// ------------------------------------------------------------ tensor cores

// acc * 2^E as a double, built with integer operations only (GB300 runs
// int->double conversion and FP64 multiplies on its narrow FP64 pipe, which
// made them the cost of the recombination).  Valid when acc != 0 and the
// result is a normal number; the caller checks the exponent range.
__device__ __forceinline__ double int_times_pow2(int acc, int E) {
  const unsigned a = acc < 0 ? 0u - (unsigned)acc : (unsigned)acc;
  const int e2 = 31 - __clz(a);                                   // a = 1.f * 2^e2
  const unsigned long long mant = ((unsigned long long)a << (52 - e2)) & 0xfffffffffffffull;
  const unsigned long long bits = ((unsigned long long)(acc < 0) << 63) |
                                  ((unsigned long long)(unsigned)(e2 + E + 1023) << 52) | mant;
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, unsigned parity, volatile int *abort_flag) {
  for (unsigned i = 0; i < kMbarPollLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *abort_flag) return false;
  }
  atomicOr(&g_split_status, kErrMbarTimeout);
  *abort_flag = 1;
  return false;
}

__global__ void __launch_bounds__(SPLIT_THREADS, 1)
    ozaki_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, SplitArgs p) {
  extern __shared__ unsigned char smem_dyn[];
  const uint32_t raw = smem_u32(smem_dyn);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  unsigned char *base = smem_dyn + pad;                           // 1024-byte aligned stage ring
  uint64_t *full = reinterpret_cast<uint64_t *>(base + STAGES * STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *acc_full = empty + STAGES;
  uint64_t *acc_empty = acc_full + 2;
  uint64_t *done = acc_empty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  __shared__ double colscale[TN];
  __shared__ int colexp[TN];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Tile order: CTAs launch in linear order; consecutive CTAs walk groups of
  // kRasterN column tiles row tile by row tile, so the CTAs resident at one
  // time share few A and B slices (L2 reuse across the wave).
  int m0, n0;
  {
    const int L = blockIdx.x + blockIdx.y * gridDim.x, Mt = gridDim.x, Nt = gridDim.y;
    const int g = L / (kRasterN * Mt), loc = L - g * kRasterN * Mt;
    const int gw = (Nt - g * kRasterN < kRasterN) ? Nt - g * kRasterN : kRasterN;
    m0 = (loc / gw) * TM;
    n0 = (g * kRasterN + loc % gw + p.nt0) * TN;
  }
  const int nkb = p.Kp / KB;
  const int nchunk = (nkb + KCHUNK_BLOCKS - 1) / KCHUNK_BLOCKS;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], 1); }
    for (int i = 0; i < 2; ++i) { mbar_init(&acc_full[i], 1); mbar_init(&acc_empty[i], EPI_WARPS * 32); }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  for (int c = threadIdx.x; c < TN; c += SPLIT_THREADS) {
    const int col = n0 + c;
    colscale[c] = (col < p.N) ? ldexp(1.0, p.exB[col]) : 0.0;
    colexp[c] = (col < p.N) ? p.exB[col] : 0;
  }
  if (warp == 1) tmem_alloc(tmem_slot, 2 * TN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tmap(&tmA);
      prefetch_tmap(&tmB);
      long it = 0;
      bool ok = true;
      for (int d = p.s - 1; d >= 0 && ok; --d)
        for (int t = 0; t <= d && ok; ++t) {
          const int u = d - t;
          for (int kb = 0; kb < nkb && ok; ++kb, ++it) {
            const int st = (int)(it % STAGES);
            const unsigned ph = (unsigned)((it / STAGES) & 1);
            if (!wait_or_abort(&empty[st], ph ^ 1u, abort_flag)) { ok = false; break; }
            unsigned char *sa = base + st * STAGE_BYTES;
            mbar_arrive_expect_tx(&full[st], STAGE_BYTES);
            tma_load_2d(sa, &tmA, &full[st], kb * KB, t * p.Mp + m0);
            tma_load_2d(sa + TM * KB * 2, &tmB, &full[st], kb * KB, u * p.Np + n0);
          }
        }
      // drain: every load issued has landed before the CTA can exit
      for (long j = (it > STAGES ? it - STAGES : 0); j < it; ++j)
        wait_or_abort(&full[j % STAGES], (unsigned)((j / STAGES) & 1), abort_flag);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_f16_f32(TM, TN);
      long it = 0, cc = 0;
      bool ok = true;
      for (int d = p.s - 1; d >= 0 && ok; --d)
        for (int t = 0; t <= d && ok; ++t)
          for (int ch = 0; ch < nchunk && ok; ++ch, ++cc) {
            const int buf = (int)(cc & 1);
            if (!wait_or_abort(&acc_empty[buf], (unsigned)(((cc >> 1) & 1) ^ 1), abort_flag)) { ok = false; break; }
            tc_fence_after();
            const uint32_t dt = tmem + (uint32_t)(buf * TN);
            const int kb0 = ch * KCHUNK_BLOCKS;
            const int kb1 = (kb0 + KCHUNK_BLOCKS < nkb) ? kb0 + KCHUNK_BLOCKS : nkb;
            for (int kb = kb0; kb < kb1; ++kb, ++it) {
              const int st = (int)(it % STAGES);
              if (!wait_or_abort(&full[st], (unsigned)((it / STAGES) & 1), abort_flag)) { ok = false; break; }
              tc_fence_after();
              const uint32_t sa = smem_u32(base + st * STAGE_BYTES);
              const uint64_t da = sw128_kmajor_desc(sa);
              const uint64_t db = sw128_kmajor_desc(sa + TM * KB * 2);
#pragma unroll
              for (int kk = 0; kk < KB / 16; ++kk)   // K = 16 per MMA: 32 bytes along the swizzled row
                mma_f16(dt, da + (uint64_t)(2 * kk), db + (uint64_t)(2 * kk), idesc, (kb > kb0 || kk > 0) ? 1u : 0u);
              mma_commit(&empty[st]);
            }
            if (!ok) break;
            mma_commit(&acc_full[buf]);
          }
      // all issued MMAs complete before tensor memory is released
      mma_commit(done);
      wait_or_abort(done, 0, abort_flag);
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2..17)
    const int q = warp & 3;                 // tensor-memory lane quarter of this warp
    const int h = (warp - 2) >> 2;          // column quarter of the tile
    const int row = q * 32 + lane;
    const int gm = m0 + row;
    const bool row_ok = gm < p.M;
    const double rowpow = row_ok ? p.alpha : 0.0;
    const int rexp = row_ok ? p.exA[gm] : 0;
    int acc[EPI_COLS];
#pragma unroll
    for (int c = 0; c < EPI_COLS; ++c) acc[c] = 0;
    long cc = 0;
    bool first = true, ok = true;
    for (int d = p.s - 1; d >= 0 && ok; --d) {
      for (int t = 0; t <= d && ok; ++t)
        for (int ch = 0; ch < nchunk; ++ch, ++cc) {
          const int buf = (int)(cc & 1);
          int okw = 1;
          if (lane == 0) okw = wait_or_abort(&acc_full[buf], (unsigned)((cc >> 1) & 1), abort_flag) ? 1 : 0;
          okw = __shfl_sync(0xffffffffu, okw, 0);
          if (!okw) { ok = false; break; }
          tc_fence_after();
#pragma unroll
          for (int cb = 0; cb < EPI_COLS / 16; ++cb) {
            uint32_t r[16];
            tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * TN + h * EPI_COLS + cb * 16), r);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; ++j) acc[cb * 16 + j] += __float2int_rn(__uint_as_float(r[j]));
          }
          tc_fence_before();
          mbar_arrive(&acc_empty[buf]);
        }
      if (!ok) break;
      // diagonal d complete: C (+)= alpha 2^(ea - 7(d+2)) acc 2^(eb).  Every
      // diagonal after the first (and the first too when beta = 1) is added
      // with fire-and-forget FP64 reductions in L2: the epilogue does not wait
      // for C, so the MMAs of the next diagonal keep running.  Each element
      // belongs to one thread, whose same-address operations stay in program
      // order, so C sees the same sequence of rounded additions as a
      // load/add/store would produce.
      const double fr = ldexp(rowpow, rexp - kSliceBits * (d + 2));
      // mode 0: reduction; 1: plain store (first diagonal, beta = 0);
      // 2: C = beta C + v with C read in batches of 8 loads before any store
      const int mode = (!first || p.beta == 1.0) ? 0 : (p.beta == 0.0 ? 1 : 2);
      const int ncol = row_ok ? p.N - (n0 + h * EPI_COLS) : 0;   // valid columns of this thread
      const size_t ldc = (size_t)p.ldc;
      double *cp = p.C + gm + (size_t)(n0 + h * EPI_COLS) * ldc;
      const double *cs = colscale + h * EPI_COLS;
      const int *ce = colexp + h * EPI_COLS;
      // alpha = +-2^k: v = (acc * fr) * cs is acc * 2^(rE + eb) exactly while
      // acc * fr and the result are normal numbers; then v is assembled from
      // integers (same value), otherwise computed in FP64 as written
      const int rE = rexp - kSliceBits * (d + 2) + p.alpha_exp;
      const bool pow2 = p.alpha_pow2 != 0;
      const bool aneg = p.alpha < 0.0;
      auto term = [&](int c) -> double {
        const int a = aneg ? -acc[c] : acc[c];
        if (pow2) {
          if (a == 0) return aneg ? -0.0 : 0.0;
          const unsigned ua = a < 0 ? 0u - (unsigned)a : (unsigned)a;
          const int e2 = 31 - __clz(ua);
          const int e_mid = e2 + rE, e_out = e_mid + ce[c];
          if (e_mid >= -1022 && e_mid <= 1023 && e_out >= -1022 && e_out <= 1023) return int_times_pow2(a, rE + ce[c]);
        }
        return (double)acc[c] * fr * cs[c];
      };
      if (mode == 0) {
#pragma unroll
        for (int c = 0; c < EPI_COLS; ++c) {
          if (c < ncol) red_add_f64(cp, term(c));
          cp += ldc;
          acc[c] = 0;
        }
      } else {
#pragma unroll
        for (int c0 = 0; c0 < EPI_COLS; c0 += 8) {
          double old[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) old[j] = (mode == 2 && c0 + j < ncol) ? cp[j * ldc] : 0.0;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const double v = term(c0 + j);
            if (c0 + j < ncol) cp[j * ldc] = (mode == 2) ? fma(p.beta, old[j], v) : v;
            acc[c0 + j] = 0;
          }
          cp += 8 * ldc;
        }
      }
      first = false;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, 2 * TN);
  }
}

// ---------------------------------------------------------------- host side
static int ceil_to(int x, int m) { return (x + m - 1) / m * m; }

// Exponents and slices of both operands (into the split slots) and the
// tensor maps over them; K <= 16384 (one exact int32 accumulation).
void dev_dgemm_split_prepare(int TA, int TB, int M, int N, int K, const double *A, int lda, const double *B, int ldb,
                             int s, SplitPlan *plan, cudaStream_t st, int slot_set) {
  Context &c = ctx();
  const int Mp = ceil_to(M, TM), Np = ceil_to(N, TN), Kp = ceil_to(K, KB);
  const int sa = slot_set ? kBufS3 : kBufS0, sb = slot_set ? kBufS4 : kBufS1, se = slot_set ? kBufS5 : kBufS2;
  __half *As = static_cast<__half *>(c.buffer(sa, sizeof(__half) * (size_t)s * Mp * Kp));
  __half *Bs = static_cast<__half *>(c.buffer(sb, sizeof(__half) * (size_t)s * Np * Kp));
  int *ex = static_cast<int *>(c.buffer(se, sizeof(int) * (size_t)(Mp + Np)));
  int *exA = ex, *exB = ex + Mp;
  // op(A)(i,k): TA==N -> A[i + k lda];  TA==T -> A[k + i lda]
  const long ars = (TA == kNoTrans) ? 1 : lda, aks = (TA == kNoTrans) ? lda : 1;
  // op(B)(k,j) seen as vector j over k: TB==N -> B[k + j ldb];  TB==T -> B[j + k ldb]
  const long brs = (TB == kNoTrans) ? ldb : 1, bks = (TB == kNoTrans) ? 1 : ldb;
  vec_exp_kernel<<<aks == 1 ? (M + 7) / 8 : (M + 31) / 32, 256, 0, st>>>(M, K, A, ars, aks, exA);
  vec_exp_kernel<<<bks == 1 ? (N + 7) / 8 : (N + 31) / 32, 256, 0, st>>>(N, K, B, brs, bks, exB);
  slice_kernel<<<dim3(Kp / 32, Mp / 32), 256, 0, st>>>(M, K, Mp, Kp, s, A, ars, aks, exA, As);
  slice_kernel<<<dim3(Kp / 32, Np / 32), 256, 0, st>>>(N, K, Np, Kp, s, B, brs, bks, exB, Bs);
  note_launch(4);
  if (!encode_tmap_2d(&plan->tA, As, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, Kp, (uint64_t)s * Mp, Kp, KB, TM,
                      CU_TENSOR_MAP_SWIZZLE_128B) ||
      !encode_tmap_2d(&plan->tB, Bs, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, Kp, (uint64_t)s * Np, Kp, KB, TN,
                      CU_TENSOR_MAP_SWIZZLE_128B)) {
    fprintf(stderr, "atlas_gb300: split dgemm: tensor map encoding failed\n");
    abort();
  }
  SplitArgs &a = plan->a;
  a.M = M; a.N = N; a.Mp = Mp; a.Np = Np; a.Kp = Kp; a.s = s; a.nt0 = 0;
  a.exA = exA; a.exB = exB;
}

// C[:, col range] = alpha*op(A)op(B) + beta*C for the output column tiles
// [t0, t1) of a prepared product (tiles of 256 columns; t1 clipped).
void dev_dgemm_split_run(const SplitPlan &plan, int t0, int t1, double alpha, double beta, double *C, int ldc,
                         cudaStream_t st) {
  const int nt = plan.a.Np / TN;
  if (t1 > nt) t1 = nt;
  if (t0 >= t1) return;
  SplitArgs a = plan.a;
  a.alpha = alpha; a.beta = beta; a.C = C; a.ldc = ldc; a.nt0 = t0;
  {
    int e = 0;
    const double m = frexp(alpha, &e);                // alpha = m 2^e, |m| in [0.5, 1)
    a.alpha_pow2 = (m == 0.5 || m == -0.5) ? 1 : 0;
    a.alpha_exp = e - 1;
  }
  ATLG_CHECK(cudaFuncSetAttribute(ozaki_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SPLIT_SMEM));
  ozaki_tc_kernel<<<dim3(a.Mp / TM, t1 - t0), SPLIT_THREADS, SPLIT_SMEM, st>>>(plan.tA, plan.tB, a);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

static void split_one(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
                      int ldb, double beta, double *C, int ldc, int s, cudaStream_t st) {
  SplitPlan plan;
  dev_dgemm_split_prepare(TA, TB, M, N, K, A, lda, B, ldb, s, &plan, st);
  dev_dgemm_split_run(plan, 0, plan.a.Np / TN, alpha, beta, C, ldc, st);
}

void dev_dgemm_split(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
                     int ldb, double beta, double *C, int ldc, int nslices, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  if (nslices < 1) nslices = 1;
  if (nslices > 8) nslices = 8;
  if (alpha == 0.0 || K <= 0) {
    dev_gescal(M, N, beta, C, ldc, st);
    return;
  }
  // int32 sums stay exact for K <= 16384 (8 pairs x 16 chunks x 2^24 < 2^31)
  const int kmax = 16384;
  for (int k0 = 0; k0 < K; k0 += kmax) {
    const int kk = (K - k0 < kmax) ? K - k0 : kmax;
    const double *Ak = (TA == kNoTrans) ? A + (size_t)k0 * lda : A + k0;
    const double *Bk = (TB == kNoTrans) ? B + k0 : B + (size_t)k0 * ldb;
    split_one(TA, TB, M, N, kk, alpha, Ak, lda, Bk, ldb, k0 == 0 ? beta : 1.0, C, ldc, nslices, st);
  }
}

unsigned split_status_read_and_clear() {
  unsigned v = 0, z = 0;
  ATLG_CHECK(cudaMemcpyFromSymbol(&v, g_split_status, sizeof(v)));
  if (v) ATLG_CHECK(cudaMemcpyToSymbol(g_split_status, &z, sizeof(z)));
  return v;
}

}  // namespace atlg
