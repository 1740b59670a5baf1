// tf32.cu -- FP32 GEMM update C += alpha * A * B (all column-major, no
// transposes) on the fifth-generation tensor cores with the 3xTF32 split:
//   a = a_hi + a_lo,  a_hi = TF32(a) (round to nearest),  a_lo = a - a_hi,
//   a*b ~= a_hi*b_hi + a_hi*b_lo + a_lo*b_hi,
// which keeps FP32-level accuracy (the dropped a_lo*b_lo term is ~2^-22
// relative) on tcgen05.mma kind::tf32.  The three products are one MMA
// chain over a concatenated K: A' = [A_lo | A_hi | A_hi], B' = [B_hi; B_lo; B_hi],
// the two small products first.  The order matters: the chain's FP32
// accumulator loses precision in proportion to its magnitude at each MMA,
// and adding the small products to the small partial sum before the large
// ones halved the refinement steps of the mixed solver at kappa = 1e6 (18 ->
// 10 at n = 16384) and cut the factor's scaled residual by ~30%, measured
// against the large-products-first order.
//
// No reference counterpart: it is the FP32 factorization inside the
// mixed-precision solver (mixed.cu) -- the "TF32 via tcgen05" factor.  The
// reference-semantics clapack_sgetrf keeps the FFMA GEMM of gemm.cu.
//
// Kernel: one 256 x 128 tile of C per CTA, 10 warps: warp 0 TMA producer
// (K-major 128-byte-swizzled tiles of A' and B', 32 FP32 per row, 2 x 48 KB
// stages), warp 1 tensor-memory allocation (256 columns) and MMA issue
// (K = 8 per instruction, two 128-row accumulators), warps 2-9 stream the
// accumulators out of tensor memory and update C in place (each thread one
// row, 128 columns; the tile of C is prefetched into L2 while the MMAs run).  Two CTAs fit per SM, so
// one CTA's epilogue (the C read-modify-write, which bounds the LU update)
// overlaps the other's MMAs.  All waits are bounded.
#include "common.cuh"
#include "context.cuh"
#include "tc.cuh"
#include "tf32.cuh"

namespace atlg {

__device__ unsigned g_tf32_status;

// A CTA's tile of C is 256 rows x 128 columns, two 128 x 128 accumulators in
// tensor memory (rows 0-127 in columns 0-127, rows 128-255 in 128-255): each
// column of the tile is 1 KB of contiguous C, the unit the read-modify-write
// moves (a 128 x 256 tile gave 512-byte pieces).
constexpr int XT_M = 256, XT_MM = 128, XT_N = 128, XT_KB = 32;   // 32 FP32 = one 128-byte swizzle row
constexpr int XT_TMEM = 2 * XT_N;                                 // tensor-memory columns
constexpr int XT_STAGES = 2;
constexpr int XT_STAGE_BYTES = (XT_M + XT_N) * XT_KB * 4;   // 48 KB
constexpr int XT_EPI_WARPS = 8;
constexpr int XT_THREADS = 64 + XT_EPI_WARPS * 32;
constexpr int XT_SMEM = XT_STAGES * XT_STAGE_BYTES + 1024 + 128;

// A' [i][k'] (Rp rows, ld = 3*Kp):  k' = [0,Kp): lo   [Kp,2Kp): hi   [2Kp,3Kp): hi
// for In(r, k) = In[r*rs + k*ks]; zero outside R x K.  `lo_mid` selects the
// B' order [hi; lo; hi] instead.
__global__ void __launch_bounds__(256) pack3_kernel(int R, int K, int Rp, int Kp, const float *__restrict__ In,
                                                    long rs, long ks, int lo_mid, float *__restrict__ Out) {
  const long total = (long)Rp * Kp;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int k = (int)(e % Kp), r = (int)(e / Kp);
    float v = 0.f;
    if (r < R && k < K) v = In[(size_t)r * rs + (size_t)k * ks];
    const float hi = tf32_rna(v);
    const float lo = v - hi;
    float *o = Out + (size_t)r * 3 * Kp;
    o[k] = lo_mid ? hi : lo;
    o[Kp + k] = lo_mid ? lo : hi;
    o[2 * Kp + k] = hi;
  }
}

struct XtArgs {
  int M, N, K3;
  float alpha;
  float *C;
  int ldc;
  int bulk_pf;   // C 16-byte aligned with ldc a multiple of 4: columns prefetched as bulk ranges
};

__device__ __forceinline__ bool xt_wait(uint64_t *bar, unsigned parity, volatile int *abort_flag) {
  for (unsigned i = 0; i < kMbarPollLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *abort_flag) return false;
  }
  atomicOr(&g_tf32_status, kErrMbarTimeout);
  *abort_flag = 1;
  return false;
}

__global__ void __launch_bounds__(XT_THREADS, 2)
    tf32x3_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, XtArgs p) {
  extern __shared__ unsigned char smem_dyn[];
  const uint32_t raw = smem_u32(smem_dyn);
  unsigned char *base = smem_dyn + (((raw + 1023u) & ~1023u) - raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(base + XT_STAGES * XT_STAGE_BYTES);
  uint64_t *empty = full + XT_STAGES;
  uint64_t *acc_full = empty + XT_STAGES;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_full + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * XT_M, n0 = blockIdx.y * XT_N;
  const int nkb = p.K3 / XT_KB;

  if (threadIdx.x == 0) {
    for (int i = 0; i < XT_STAGES; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], 1); }
    mbar_init(acc_full, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, XT_TMEM);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      prefetch_tmap(&tmA);
      prefetch_tmap(&tmB);
      int kb = 0;
      for (; kb < nkb; ++kb) {
        const int st = kb % XT_STAGES;
        if (!xt_wait(&empty[st], (unsigned)(((kb / XT_STAGES) & 1) ^ 1), abort_flag)) break;
        unsigned char *sa = base + st * XT_STAGE_BYTES;
        mbar_arrive_expect_tx(&full[st], XT_STAGE_BYTES);
        tma_load_2d(sa, &tmA, &full[st], kb * XT_KB, m0);
        tma_load_2d(sa + XT_M * XT_KB * 4, &tmB, &full[st], kb * XT_KB, n0);
      }
      for (int j = (kb > XT_STAGES ? kb - XT_STAGES : 0); j < kb; ++j)
        xt_wait(&full[j % XT_STAGES], (unsigned)((j / XT_STAGES) & 1), abort_flag);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32 (2 at bits 7-9 and 10-12), K-major
      const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(XT_N >> 3) << 17) |
                             ((uint32_t)(XT_MM >> 4) << 24);
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb % XT_STAGES;
        if (!xt_wait(&full[st], (unsigned)((kb / XT_STAGES) & 1), abort_flag)) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(base + st * XT_STAGE_BYTES);
        const uint64_t da = sw128_kmajor_desc(sa);                             // rows 0-127
        const uint64_t da1 = sw128_kmajor_desc(sa + XT_MM * XT_KB * 4);        // rows 128-255
        const uint64_t db = sw128_kmajor_desc(sa + XT_M * XT_KB * 4);
#pragma unroll
        for (int kk = 0; kk < XT_KB / 8; ++kk) {   // K = 8 per MMA: 32 bytes along the swizzled row
          asm volatile(
              "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
              "l"(da + (uint64_t)(2 * kk)), "l"(db + (uint64_t)(2 * kk)), "r"(idesc),
              "r"((kb > 0 || kk > 0) ? 1u : 0u)
              : "memory");
          asm volatile(
              "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem + (uint32_t)XT_N),
              "l"(da1 + (uint64_t)(2 * kk)), "l"(db + (uint64_t)(2 * kk)), "r"(idesc),
              "r"((kb > 0 || kk > 0) ? 1u : 0u)
              : "memory");
        }
        mma_commit(&empty[st]);
      }
      mma_commit(acc_full);   // arrives once every MMA issued above has completed
    }
  } else {
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;            // which accumulator: rows h*128 .. h*128+127 of the tile
    const int row = h * XT_MM + q * 32 + lane;
    const int gm = m0 + row;
    const bool rok = gm < p.M;
    float *crow = p.C + gm;
    // the tile's C into L2 while the MMAs run: the epilogue's reads then
    // come from L2 instead of waiting on HBM 16 loads at a time.  Aligned C:
    // each thread one bulk prefetch of one column's rows of the tile; else a
    // warp-wide prefetch per 128-byte line
    if (p.bulk_pf) {
      const int t = (warp - 2) * 32 + lane;   // warps 2-5: one column each
      const int gn = n0 + t;
      const int rows = (p.M - m0 < XT_M ? p.M - m0 : XT_M) & ~3;
      if (t < XT_N && gn < p.N && rows > 0)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p.C + m0 + (size_t)gn * p.ldc),
                     "r"(rows * 4)
                     : "memory");
    } else if (rok) {
      for (int j = 0; j < XT_N; ++j) {
        const int gn = n0 + j;
        if (gn < p.N) prefetch_l2(crow + (size_t)gn * p.ldc);
      }
    }
    // a tile inside C on both sides needs no bounds tests
    const bool inner = (m0 + XT_M <= p.M) && (n0 + XT_N <= p.N);
    float *cbase = crow + (size_t)n0 * p.ldc;
    // C is read in batches of 16 columns, two batches ahead of the one being
    // finished (the first two before the accumulator is ready), so the
    // read-modify-write is bandwidth- rather than latency-bound
    auto load_batch = [&](float (&cv)[16], int cb) {
      if (inner) {
        const float *cp = cbase + (size_t)(cb * 16) * p.ldc;
#pragma unroll
        for (int j = 0; j < 16; ++j) cv[j] = __ldcs(cp + (size_t)j * p.ldc);
        return;
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int gn = n0 + cb * 16 + j;
        cv[j] = (rok && gn < p.N) ? __ldcs(crow + (size_t)gn * p.ldc) : 0.f;
      }
    };
    float cv0[16], cv1[16];
    load_batch(cv0, 0);
    load_batch(cv1, 1);
    int okw = 1;
    if (lane == 0) okw = xt_wait(acc_full, 0, abort_flag) ? 1 : 0;
    okw = __shfl_sync(0xffffffffu, okw, 0);
    if (okw) {
      tc_fence_after();
#pragma unroll
      for (int cb = 0; cb < 8; ++cb) {
        float (&cv)[16] = (cb & 1) ? cv1 : cv0;
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 128 + cb * 16), r);
        tmem_wait_ld();
        float out[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) out[j] = fmaf(p.alpha, __uint_as_float(r[j]), cv[j]);
        if (cb + 2 < 8) load_batch(cv, cb + 2);
        if (inner) {
          float *cp = cbase + (size_t)(cb * 16) * p.ldc;
#pragma unroll
          for (int j = 0; j < 16; ++j) __stcs(cp + (size_t)j * p.ldc, out[j]);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int gn = n0 + cb * 16 + j;
            if (rok && gn < p.N) __stcs(crow + (size_t)gn * p.ldc, out[j]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, XT_TMEM);
  }
}

static int ceil_to(int x, int m) { return (x + m - 1) / m * m; }

static int grid_for(long work) {
  long b = (work + 255) / 256;
  if (b > 16L * 152) b = 16L * 152;
  return b < 1 ? 1 : (int)b;
}

void dev_sgemm_tf32x3_pack_a(int M, int K, const float *A, int lda, float *Ap, cudaStream_t st) {
  const int Mp = ceil_to(M, XT_M), Kp = ceil_to(K, XT_KB);
  pack3_kernel<<<grid_for((long)Mp * Kp), 256, 0, st>>>(M, K, Mp, Kp, A, 1, lda, 0, Ap);
  note_launch();
}
void dev_sgemm_tf32x3_pack_b(int K, int N, const float *B, int ldb, float *Bp, cudaStream_t st) {
  const int Np = ceil_to(N, XT_N), Kp = ceil_to(K, XT_KB);
  pack3_kernel<<<grid_for((long)Np * Kp), 256, 0, st>>>(N, K, Np, Kp, B, ldb, 1, 1, Bp);
  note_launch();
}
// The same packing for exactly N rows (no padding rows written): a caller
// that packs one operand in parts, each at its own row offset of Bp.
void dev_sgemm_tf32x3_pack_b_rows(int K, int N, const float *B, int ldb, float *Bp, cudaStream_t st) {
  if (N <= 0) return;
  const int Kp = ceil_to(K, XT_KB);
  pack3_kernel<<<grid_for((long)N * Kp), 256, 0, st>>>(N, K, N, Kp, B, ldb, 1, 1, Bp);
  note_launch();
}
size_t tf32x3_packed_floats(int rows, int K, bool b_operand) {
  return (size_t)ceil_to(rows, b_operand ? XT_N : XT_M) * 3 * (size_t)ceil_to(K, XT_KB);
}

// C[M x N] += alpha * A * B from packed operands: Ap from pack_a (rows of A),
// Bp from pack_b starting `boff` rows (columns of B) into the packing.
void dev_sgemm_tf32x3_packed(int M, int N, int K, float alpha, const float *Ap, const float *Bp, int b_rows_total,
                             int boff, float *C, int ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  const int Kp = ceil_to(K, XT_KB), K3 = 3 * Kp;
  const int Mp = ceil_to(M, XT_M);
  const int Nrows = ceil_to(b_rows_total, XT_N);
  CUtensorMap tA, tB;
  const float *Bsub = Bp + (size_t)boff * K3;
  if (!encode_tmap_2d(&tA, Ap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, K3, Mp, K3, XT_KB, XT_M,
                      CU_TENSOR_MAP_SWIZZLE_128B) ||
      !encode_tmap_2d(&tB, Bsub, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, K3, Nrows - boff, K3, XT_KB, XT_N,
                      CU_TENSOR_MAP_SWIZZLE_128B)) {
    fprintf(stderr, "atlas_gb300: tf32x3 update: tensor map encoding failed\n");
    abort();
  }
  XtArgs a;
  a.M = M; a.N = N; a.K3 = K3; a.alpha = alpha; a.C = C; a.ldc = ldc;
  a.bulk_pf = ((reinterpret_cast<uintptr_t>(C) & 15) == 0 && (ldc & 3) == 0) ? 1 : 0;
  ATLG_CHECK(cudaFuncSetAttribute(tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, XT_SMEM));
  tf32x3_kernel<<<dim3(Mp / XT_M, (N + XT_N - 1) / XT_N), XT_THREADS, XT_SMEM, st>>>(tA, tB, a);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

unsigned tf32_status_read_and_clear() {
  unsigned v = 0, z = 0;
  ATLG_CHECK(cudaMemcpyFromSymbol(&v, g_tf32_status, sizeof(v)));
  if (v) ATLG_CHECK(cudaMemcpyToSymbol(g_tf32_status, &z, sizeof(z)));
  return v;
}

}  // namespace atlg
