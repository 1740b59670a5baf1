// gemm.cu -- C = alpha*op(A)*op(B) + beta*C for FP64 (DGEMM) and FP32 (SGEMM)
// on GB300, column-major, any op/shape/leading dimension.
//
// Replaces the reference's AMM GEMM stack: ATL_dammm recursion and shape
// dispatch (AtlasBase/Clint/atlas-ammm.base:15624, 17707-17811), the
// access-major copy/pack routines with alpha/beta (Students/trmm-micro-cpg.base:
// 15-120, Clint/atlas-mmcpy.base) and the register-blocked ammkern_t kernels
// (AtlasBase/kernel/ClintWhaley/*.S).
//
// GB300 design.  FP64 on GB300 runs on the CUDA-core DFMA pipe (measured
// 1.19 TFLOP/s for DFMA against 1.05 TFLOP/s for FP64 mma.sync), so the FP64
// kernel is a register-tiled DFMA kernel; the same template with FFMA serves
// FP32.  Operand tiles are staged global -> shared by TMA tensor loads
// (cp.async.bulk.tensor.2d, zero fill at the matrix edges) into a STAGES-deep
// ring completed on mbarriers; a matrix TMA cannot address (base not 16-byte
// aligned, leading dimension not a multiple of 16 bytes) takes a cp.async
// zero-fill pipeline with the same shared-memory layout.  alpha/beta are
// fused into the epilogue (beta == 0 never reads C).  The tile shape is picked
// per call to balance the CTAs over the 152 SMs.
#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"

namespace atlg {

__device__ unsigned g_gemm_status;

template <typename T, int BM, int BN, int BK, int TM, int TN, int NT, int STAGES, int TA, int TB,
          bool USE_TMA>
struct GemmKernel {
  static constexpr int A_ELEMS = BM * BK;
  static constexpr int B_ELEMS = BK * BN;
  static constexpr int STAGE_ELEMS = A_ELEMS + B_ELEMS;
  static constexpr int SMEM_BYTES = STAGES * STAGE_ELEMS * (int)sizeof(T) + 64;
  static constexpr int GX = BM / TM;   // threads along m
  static constexpr int GY = BN / TN;   // threads along n
  static_assert(GX * GY == NT, "thread grid");
  static_assert(A_ELEMS % NT == 0 && B_ELEMS % NT == 0, "loader split");
};

// op(A)(m,k) inside a stage:  TA==N -> [k][m],  TA==T -> [m][k]
template <int TA, int BM, int BK>
__device__ __forceinline__ int a_idx(int m, int k) {
  return TA == kNoTrans ? k * BM + m : m * BK + k;
}
// op(B)(k,n) inside a stage:  TB==N -> [n][k],  TB==T -> [k][n]
template <int TB, int BN, int BK>
__device__ __forceinline__ int b_idx(int k, int n) {
  return TB == kNoTrans ? n * BK + k : k * BN + n;
}

// SUB: C -= op(A)*op(B) (alpha = -1, beta = 1, the LU's trailing update):
// the accumulators start from C and take fma(-a, b, acc), so the epilogue is
// a store -- no FP64 instruction besides the K DFMAs per element, where the
// general epilogue spends two (alpha*acc, then beta*c + v) per K = 64 tile:
// 3% of an FP64 pipe that bounds the kernel.
template <typename T, int BM, int BN, int BK, int TM, int TN, int NT, int STAGES, int TA, int TB,
          bool USE_TMA, bool SUB = false>
__global__ void __launch_bounds__(NT)
    gemm_kernel(int M, int N, int K, T alpha, const T *__restrict__ A, int lda,
                const T *__restrict__ B, int ldb, T beta, T *__restrict__ C, int ldc, int uplo, int tri,
                const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, long sA, long sB,
                long sC) {
  using KC = GemmKernel<T, BM, BN, BK, TM, TN, NT, STAGES, TA, TB, USE_TMA>;
  if (!USE_TMA && blockIdx.z) {   // batched products (pointer arithmetic only on the cp.async path)
    A += blockIdx.z * sA;
    B += blockIdx.z * sB;
    C += blockIdx.z * sC;
  }
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + STAGES * KC::STAGE_ELEMS * sizeof(T));

  const int tid = threadIdx.x;
  const int m0 = blockIdx.x * BM;
  const int n0 = blockIdx.y * BN;
  // triangle-masked update (SYRK): tiles wholly outside the triangle exit
  if ((uplo == kLower && m0 + BM <= n0) || (uplo == kUpper && n0 + BN <= m0)) return;
  // triangular operand (TRMM): only the k-tiles that meet the triangle
  int kt0 = 0, kt1 = (K + BK - 1) / BK;
  if (tri) {
    const bool up = (tri & kTriUpper) != 0;
    if ((tri & kTriWhich) == kTriA) {          // op(A) upper: k >= m;  lower: k <= m
      if (up) kt0 = m0 / BK;
      else kt1 = ((K < m0 + BM ? K : m0 + BM) + BK - 1) / BK;
    } else {                                    // op(B) upper: k <= n;  lower: k >= n
      if (up) kt1 = ((K < n0 + BN ? K : n0 + BN) + BK - 1) / BK;
      else kt0 = n0 / BK;
    }
  }
  const int KT = kt1 - kt0;
  const int tx = tid % KC::GX, ty = tid / KC::GX;

  T acc[TM][TN];
  if (SUB) {
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = n0 + ty + j * KC::GY;
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int m = m0 + tx + i * KC::GX;
        acc[i][j] = (m < M && n < N) ? C[m + (size_t)n * ldc] : T(0);
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
  }

  auto stageA = [&](int s) { return smem + s * KC::STAGE_ELEMS; };
  auto stageB = [&](int s) { return smem + s * KC::STAGE_ELEMS + KC::A_ELEMS; };

  // ---- producers ----------------------------------------------------------
  auto issue_tma = [&](int kt, int s) {
    const unsigned bytes = KC::STAGE_ELEMS * sizeof(T);
    mbar_arrive_expect_tx(&full[s], bytes);
    const int k0 = kt * BK;
    if (TA == kNoTrans) tma_load_2d(stageA(s), &tmA, &full[s], m0, k0);
    else                tma_load_2d(stageA(s), &tmA, &full[s], k0, m0);
    if (TB == kNoTrans) tma_load_2d(stageB(s), &tmB, &full[s], k0, n0);
    else                tma_load_2d(stageB(s), &tmB, &full[s], n0, k0);
  };
  auto issue_cpasync = [&](int kt, int s) {
    const int k0 = kt * BK;
    T *sa = stageA(s), *sb = stageB(s);
#pragma unroll
    for (int e = tid; e < KC::A_ELEMS; e += NT) {
      int m, k;
      if (TA == kNoTrans) { m = e % BM; k = e / BM; } else { k = e % BK; m = e / BK; }
      const int gm = m0 + m, gk = k0 + k;
      const bool ok = gm < M && gk < K;
      const T *src = ok ? (TA == kNoTrans ? A + gm + (size_t)gk * lda : A + gk + (size_t)gm * lda) : A;
      if (sizeof(T) == 8) cp_async8(sa + e, src, ok); else cp_async4(sa + e, src, ok);
    }
#pragma unroll
    for (int e = tid; e < KC::B_ELEMS; e += NT) {
      int k, n;
      if (TB == kNoTrans) { k = e % BK; n = e / BK; } else { n = e % BN; k = e / BN; }
      const int gn = n0 + n, gk = k0 + k;
      const bool ok = gn < N && gk < K;
      const T *src = ok ? (TB == kNoTrans ? B + gk + (size_t)gn * ldb : B + gn + (size_t)gk * ldb) : B;
      if (sizeof(T) == 8) cp_async8(sb + e, src, ok); else cp_async4(sb + e, src, ok);
    }
  };

  // zero the elements of a triangular operand's stage that lie outside the
  // triangle (1 on a unit diagonal); only stages that cross the diagonal
  auto tri_mask_stage = [&](int ktg, int s) {
    const int k0 = ktg * BK;
    const bool up = (tri & kTriUpper) != 0, unit = (tri & kTriUnit) != 0;
    if ((tri & kTriWhich) == kTriA) {
      if (!(k0 < m0 + BM && m0 < k0 + BK)) return;
      T *sa = stageA(s);
#pragma unroll 1
      for (int e = tid; e < KC::A_ELEMS; e += NT) {
        int m, k;
        if (TA == kNoTrans) { m = e % BM; k = e / BM; } else { k = e % BK; m = e / BK; }
        const int gm = m0 + m, gk = k0 + k;
        if (up ? gk < gm : gk > gm) sa[e] = T(0);
        else if (unit && gk == gm) sa[e] = T(1);
      }
    } else {
      if (!(k0 < n0 + BN && n0 < k0 + BK)) return;
      T *sb = stageB(s);
#pragma unroll 1
      for (int e = tid; e < KC::B_ELEMS; e += NT) {
        int k, n;
        if (TB == kNoTrans) { k = e % BK; n = e / BK; } else { n = e % BN; k = e / BN; }
        const int gn = n0 + n, gk = k0 + k;
        if (up ? gk > gn : gk < gn) sb[e] = T(0);
        else if (unit && gk == gn) sb[e] = T(1);
      }
    }
    __syncthreads();
  };

  if (USE_TMA) {
    if (tid == 0) {
      prefetch_tmap(&tmA);
      prefetch_tmap(&tmB);
      for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int s = 0; s < STAGES && s < KT; ++s) issue_tma(kt0 + s, s);
  } else {
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
      if (s < KT) issue_cpasync(kt0 + s, s);
      cp_async_commit();
    }
  }

  bool failed = false;
  for (int kt = 0; kt < KT; ++kt) {
    const int s = kt % STAGES;
    if (USE_TMA) {
      if (!mbar_wait(&full[s], (kt / STAGES) & 1, &g_gemm_status)) { failed = true; break; }
    } else {
      cp_async_wait<STAGES - 2>();
      __syncthreads();
      const int nk = kt + STAGES - 1;
      if (nk < KT) issue_cpasync(kt0 + nk, nk % STAGES);
      cp_async_commit();
    }
    if (tri) tri_mask_stage(kt0 + kt, s);
    const T *sa = stageA(s), *sb = stageB(s);
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = sa[a_idx<TA, BM, BK>(tx + i * KC::GX, k)];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = sb[b_idx<TB, BN, BK>(k, ty + j * KC::GY)];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(SUB ? -a[i] : a[i], b[j], acc[i][j]);
    }
    if (USE_TMA) {
      __syncthreads();                       // every thread is done with stage s
      if (tid == 0 && kt + STAGES < KT) {
        if (tri) fence_proxy_async();   // masked in place: order before the next TMA write
        issue_tma(kt0 + kt + STAGES, s);
      }
    }
  }
  if (!USE_TMA) cp_async_wait<0>();
  if (failed) return;

  // ---- epilogue: C = alpha*acc + beta*C --------------------------------------
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int n = n0 + ty + j * KC::GY;
    if (n >= N) continue;
    T *c = C + (size_t)n * ldc;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int m = m0 + tx + i * KC::GX;
      if (m >= M || (uplo == kLower && m < n) || (uplo == kUpper && m > n)) continue;
      if (SUB) {
        c[m] = acc[i][j];
      } else {
        const T v = alpha * acc[i][j];
        c[m] = (beta == T(0)) ? v : fma(beta, c[m], v);
      }
    }
  }
}

// ------------------------------------------------------------------ host side
template <typename T> struct DT;
template <> struct DT<double> { static constexpr CUtensorMapDataType v = CU_TENSOR_MAP_DATA_TYPE_FLOAT64; };
template <> struct DT<float>  { static constexpr CUtensorMapDataType v = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; };

template <typename T, int BM, int BN, int BK, int TM, int TN, int NT, int STAGES, int TA, int TB>
static void launch_cfg(int M, int N, int K, T alpha, const T *A, int lda, const T *B, int ldb,
                       T beta, T *C, int ldc, cudaStream_t st, bool allow_tma, int uplo, int tri,
                       const GemmOpts &o) {
  const int nb = o.batch > 1 ? o.batch : 1;
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, nb);
  CUtensorMap tmA, tmB;
  bool tma = allow_tma && nb == 1;
  if (tma) {
    // op(A) is M x K; stored TA==N as M x K (inner M), TA==T as K x M (inner K)
    if (TA == kNoTrans) tma = encode_tmap_2d(&tmA, A, DT<T>::v, sizeof(T), M, K, lda, BM, BK);
    else                tma = encode_tmap_2d(&tmA, A, DT<T>::v, sizeof(T), K, M, lda, BK, BM);
  }
  if (tma) {
    if (TB == kNoTrans) tma = encode_tmap_2d(&tmB, B, DT<T>::v, sizeof(T), K, N, ldb, BK, BN);
    else                tma = encode_tmap_2d(&tmB, B, DT<T>::v, sizeof(T), N, K, ldb, BN, BK);
  }
  if (tma) {
    using KC = GemmKernel<T, BM, BN, BK, TM, TN, NT, STAGES, TA, TB, true>;
    // C -= op(A) op(B) in FP64 without epilogue arithmetic (the LU, TRSM,
    // getrs and Cholesky updates; a SYRK's triangle mask still applies at the
    // store); FP32 keeps the general form, whose rounding the
    // reference-semantics sgetrf's pivots were checked with
    const bool sub = sizeof(T) == 8 && alpha == T(-1) && beta == T(1) && tri == 0;
    auto k = sub ? gemm_kernel<T, BM, BN, BK, TM, TN, NT, STAGES, TA, TB, true, true>
                 : gemm_kernel<T, BM, BN, BK, TM, TN, NT, STAGES, TA, TB, true, false>;
    ATLG_CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, KC::SMEM_BYTES));
    k<<<grid, NT, KC::SMEM_BYTES, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, uplo, tri, tmA, tmB, 0L, 0L,
                                        0L);
    note_launch();
  } else {
    memset(&tmA, 0, sizeof(tmA));
    memset(&tmB, 0, sizeof(tmB));
    using KC = GemmKernel<T, BM, BN, BK, TM, TN, NT, STAGES, TA, TB, false>;
    auto k = gemm_kernel<T, BM, BN, BK, TM, TN, NT, STAGES, TA, TB, false>;
    ATLG_CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, KC::SMEM_BYTES));
    k<<<grid, NT, KC::SMEM_BYTES, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, uplo, tri, tmA, tmB,
                                        o.stride_a, o.stride_b, o.stride_c);
    note_launch();
  }
  ATLG_CHECK(cudaGetLastError());
}

// Tile choice: the kernels are bound by the FP64 (or FP32) pipe, so the
// makespan is ceil(tiles/SMs) * tile area; pick the shape that minimises it
// (larger tile on ties).
static int pick_dtile(int M, int N, int nsm) {
  const int shapes[3][2] = {{64, 64}, {64, 32}, {32, 32}};
  long best = -1;
  int bi = 0;
  for (int i = 0; i < 3; ++i) {
    const long tiles = (long)((M + shapes[i][0] - 1) / shapes[i][0]) * ((N + shapes[i][1] - 1) / shapes[i][1]);
    const long span = ((tiles + nsm - 1) / nsm) * shapes[i][0] * shapes[i][1];
    if (best < 0 || span < best) { best = span; bi = i; }
  }
  return bi;
}

template <int TA, int TB>
static void dgemm_t(int M, int N, int K, double alpha, const double *A, int lda, const double *B, int ldb,
                    double beta, double *C, int ldc, cudaStream_t st, bool tma, int nsm, int uplo, int tri,
                    const GemmOpts &o) {
  // a batch spreads its products over the SMs: tile choice per product
  const int per = (o.batch > 1) ? (nsm + o.batch - 1) / o.batch : nsm;
  switch (pick_dtile(M, N, per)) {
    case 0: launch_cfg<double, 64, 64, 16, 8, 4, 128, 4, TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, tma, uplo, tri, o); break;
    case 1: launch_cfg<double, 64, 32, 16, 4, 4, 128, 4, TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, tma, uplo, tri, o); break;
    default: launch_cfg<double, 32, 32, 16, 4, 2, 128, 4, TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, tma, uplo, tri, o); break;
  }
}

template <int TA, int TB>
static void sgemm_t(int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb,
                    float beta, float *C, int ldc, cudaStream_t st, bool tma, int uplo, int tri, const GemmOpts &o) {
  launch_cfg<float, 128, 128, 16, 8, 8, 256, 4, TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, tma, uplo, tri, o);
}

__global__ void scale_kernel_d(int M, int N, double beta, double *C, int ldc) {
  const size_t total = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(e % M), n = (int)(e / M);
    double *c = C + m + (size_t)n * ldc;
    *c = (beta == 0.0) ? 0.0 : beta * *c;
  }
}
__global__ void scale_kernel_s(int M, int N, float beta, float *C, int ldc) {
  const size_t total = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(e % M), n = (int)(e / M);
    float *c = C + m + (size_t)n * ldc;
    *c = (beta == 0.0f) ? 0.0f : beta * *c;
  }
}

void dev_gescal(int M, int N, double beta, double *C, int ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0 || beta == 1.0) return;
  const size_t total = (size_t)M * N;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  scale_kernel_d<<<blocks, 256, 0, st>>>(M, N, beta, C, ldc);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}
void dev_gescal(int M, int N, float beta, float *C, int ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0 || beta == 1.0f) return;
  const size_t total = (size_t)M * N;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  scale_kernel_s<<<blocks, 256, 0, st>>>(M, N, beta, C, ldc);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}


// ------------------------------------------------------------------ GEMV
// y = alpha*op(A)*x + beta*y for the N == 1 products of TRSM, getrs and the
// refinement residual (a 64x64 GEMM tile would waste 63/64 of its work).
// op(A) = A (M x K): a CTA owns 32 rows; its 8 warps stride over the K
// columns (lanes read 32 consecutive rows, 256 B per column), and the 8
// per-warp partial sums are added in a fixed order, so the result is
// deterministic.  op(A) = A^T: a warp per output, lanes stride over the
// contiguous column, shuffle reduction in a fixed order.
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_n_kernel(int M, int K, T alpha, const T *__restrict__ A, int lda, const T *__restrict__ x, int incx,
                  T beta, T *__restrict__ y) {
  __shared__ T part[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  T acc = T(0);
  if (i < M) {
    const T *a = A + i;
    int k = w;
    // 8 columns' loads in flight per thread before their FMAs (the same
    // per-thread summation order as one column at a time)
    for (; k + 56 < K; k += 64) {
      T av[8], xv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        av[u] = a[(size_t)(k + 8 * u) * lda];
        xv[u] = x[(size_t)(k + 8 * u) * incx];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) acc = fma(av[u], xv[u], acc);
    }
    for (; k < K; k += 8) acc = fma(a[(size_t)k * lda], x[(size_t)k * incx], acc);
  }
  part[w][lane] = acc;
  __syncthreads();
  if (w == 0 && i < M) {
    T s = part[0][lane];
#pragma unroll
    for (int q = 1; q < 8; ++q) s += part[q][lane];
    const T v = alpha * s;
    y[i] = (beta == T(0)) ? v : fma(beta, y[i], v);
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    gemv_t_kernel(int M, int K, T alpha, const T *__restrict__ A, int lda, const T *__restrict__ x, int incx,
                  T beta, T *__restrict__ y) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 8 + w;
  if (i >= M) return;
  const T *a = A + (size_t)i * lda;
  T acc = T(0);
  for (int k = lane; k < K; k += 32) acc = fma(a[k], x[(size_t)k * incx], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    const T v = alpha * acc;
    y[i] = (beta == T(0)) ? v : fma(beta, y[i], v);
  }
}

// y = alpha A x + beta y for a large column-major A (NoTrans): a CTA takes a
// 2048-row x 128-column tile, so each column piece it reads is 16 KB
// contiguous (a 32-row strip per column, as gemv_n_kernel reads, leaves the
// HBM rows mostly unused); the per-tile partial sums go to `part` and one
// more kernel adds the column tiles in a fixed order.
constexpr int GV_RB = 2048, GV_CB = 128, GV_U = 4;
template <typename T>
__global__ void __launch_bounds__(256, 2)
    gemv_n_tile_kernel(int M, int K, const T *__restrict__ A, int lda, const T *__restrict__ x, int incx,
                       T *__restrict__ part, int ldp) {
  const int r0 = blockIdx.x * GV_RB, c0 = blockIdx.y * GV_CB;
  const int ce = (c0 + GV_CB < K) ? c0 + GV_CB : K;
  T acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = T(0);
  for (int c = c0; c < ce; c += GV_U) {
    T av[GV_U][8], xv[GV_U];
#pragma unroll
    for (int u = 0; u < GV_U; ++u) {
      const bool cok = c + u < ce;
      xv[u] = cok ? x[(size_t)(c + u) * incx] : T(0);
      const T *col = A + (size_t)(c + u) * lda;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = r0 + threadIdx.x + 256 * q;
        av[u][q] = (cok && i < M) ? col[i] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < GV_U; ++u)
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fma(av[u][q], xv[u], acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int i = r0 + threadIdx.x + 256 * q;
    if (i < M) part[i + (size_t)blockIdx.y * ldp] = acc[q];
  }
}
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_reduce_kernel(int M, int S, T alpha, const T *__restrict__ part, int ldp, T beta, T *__restrict__ y) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= M) return;
  T s = T(0);
  for (int g = 0; g < S; ++g) s += part[i + (size_t)g * ldp];
  const T v = alpha * s;
  y[i] = (beta == T(0)) ? v : fma(beta, y[i], v);
}

template <typename T>
static void gemv_launch(int TA, int M, int K, T alpha, const T *A, int lda, const T *x, int incx, T beta, T *y,
                        cudaStream_t st) {
  if (TA == kNoTrans && M >= GV_RB && K >= 8 * GV_CB) {
    const int S = (K + GV_CB - 1) / GV_CB;
    const int ldp = (M + 31) & ~31;
    T *part = static_cast<T *>(ctx().buffer(kBufGemv, sizeof(T) * (size_t)ldp * S));
    gemv_n_tile_kernel<T><<<dim3((M + GV_RB - 1) / GV_RB, S), 256, 0, st>>>(M, K, A, lda, x, incx, part, ldp);
    gemv_reduce_kernel<T><<<(M + 255) / 256, 256, 0, st>>>(M, S, alpha, part, ldp, beta, y);
    note_launch(2);
    ATLG_CHECK(cudaGetLastError());
    return;
  }
  if (TA == kNoTrans)
    gemv_n_kernel<T><<<(M + 31) / 32, 256, 0, st>>>(M, K, alpha, A, lda, x, incx, beta, y);
  else
    gemv_t_kernel<T><<<(M + 7) / 8, 256, 0, st>>>(M, K, alpha, A, lda, x, incx, beta, y);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

void dev_dgemv(int TA, int M, int K, double alpha, const double *A, int lda, const double *x, int incx, double beta,
               double *y, cudaStream_t st) {
  if (M <= 0) return;
  if (alpha == 0.0 || K <= 0) { dev_gescal(M, 1, beta, y, M, st); return; }
  gemv_launch<double>(TA == kNoTrans ? kNoTrans : kTrans, M, K, alpha, A, lda, x, incx, beta, y, st);
}
void dev_sgemv(int TA, int M, int K, float alpha, const float *A, int lda, const float *x, int incx, float beta,
               float *y, cudaStream_t st) {
  if (M <= 0) return;
  if (alpha == 0.0f || K <= 0) { dev_gescal(M, 1, beta, y, M, st); return; }
  gemv_launch<float>(TA == kNoTrans ? kNoTrans : kTrans, M, K, alpha, A, lda, x, incx, beta, y, st);
}

// CUDA-event bracket around one GEMM launch when profiling is on.
struct ProfScope {
  cudaStream_t st;
  double flops;
  cudaEvent_t b = nullptr;
  ProfScope(cudaStream_t s, double f) : st(s), flops(f) {
    if (ctx().prof) {
      b = ctx().event();
      ATLG_CHECK(cudaEventRecord(b, st));
    }
  }
  ~ProfScope() {
    if (b) {
      cudaEvent_t e = ctx().event();
      ATLG_CHECK(cudaEventRecord(e, st));
      ctx().recs.push_back({b, e, flops});
    }
  }
};

// ATL_gemm semantics: alpha==0 or K==0 -> C = beta*C (gescal / gezero).
void dev_dgemm(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda, const double *B,
               int ldb, double beta, double *C, int ldc, cudaStream_t st, const GemmOpts &o) {
  if (M <= 0 || N <= 0 || o.batch < 1) return;
  if (alpha == 0.0 || K <= 0) {
    for (int z = 0; z < o.batch; ++z) dev_gescal(M, N, beta, C + z * o.stride_c, ldc, st);
    return;
  }
  const bool ta = TA != kNoTrans, tb = TB != kNoTrans;
  const int nsm = o.num_sms > 0 ? o.num_sms : ctx().num_sms;
  if (N == 1 && o.allow_gemv && o.uplo == 0 && o.tri == 0 && o.batch == 1) {   // matrix-vector: x = op(B)(:,0)
    gemv_launch<double>(TA, M, K, alpha, A, lda, B, tb ? ldb : 1, beta, C, st);
    return;
  }
  ProfScope ps(st, 2.0 * M * N * K * o.batch);
  if (!ta && !tb) dgemm_t<kNoTrans, kNoTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, nsm, o.uplo, o.tri, o);
  else if (!ta && tb) dgemm_t<kNoTrans, kTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, nsm, o.uplo, o.tri, o);
  else if (ta && !tb) dgemm_t<kTrans, kNoTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, nsm, o.uplo, o.tri, o);
  else dgemm_t<kTrans, kTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, nsm, o.uplo, o.tri, o);
}

void dev_sgemm(int TA, int TB, int M, int N, int K, float alpha, const float *A, int lda, const float *B,
               int ldb, float beta, float *C, int ldc, cudaStream_t st, const GemmOpts &o) {
  if (M <= 0 || N <= 0 || o.batch < 1) return;
  if (alpha == 0.0f || K <= 0) {
    for (int z = 0; z < o.batch; ++z) dev_gescal(M, N, beta, C + z * o.stride_c, ldc, st);
    return;
  }
  const bool ta = TA != kNoTrans, tb = TB != kNoTrans;
  if (N == 1 && o.allow_gemv && o.uplo == 0 && o.tri == 0 && o.batch == 1) {
    gemv_launch<float>(TA, M, K, alpha, A, lda, B, tb ? ldb : 1, beta, C, st);
    return;
  }
  ProfScope ps(st, 2.0 * M * N * K * o.batch);
  if (!ta && !tb) sgemm_t<kNoTrans, kNoTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, o.uplo, o.tri, o);
  else if (!ta && tb) sgemm_t<kNoTrans, kTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, o.uplo, o.tri, o);
  else if (ta && !tb) sgemm_t<kTrans, kNoTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, o.uplo, o.tri, o);
  else sgemm_t<kTrans, kTrans>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, o.allow_tma, o.uplo, o.tri, o);
}

unsigned gemm_status_read_and_clear() {
  unsigned v = 0, z = 0;
  ATLG_CHECK(cudaMemcpyFromSymbol(&v, g_gemm_status, sizeof(v)));
  if (v) ATLG_CHECK(cudaMemcpyToSymbol(g_gemm_status, &z, sizeof(z)));
  return v;
}

}  // namespace atlg
