// common.cuh -- shared definitions of the GB300 (sm_103a) Level-3 / LU library.
//
// Device helpers are hand-written inline PTX for the Blackwell features the
// kernels use: mbarrier (bounded waits only), TMA tensor loads
// (cp.async.bulk.tensor), cp.async zero-fill copies and a bounded grid
// barrier.  Every wait in device code gives up after a fixed number of
// polls, records an error code in the library's device status word and lets
// the kernel return; the host reads the word after the call.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

namespace atlg {

// cblas enum values (reference ABI: AtlasBase/Clint/atlas.base:19800-19806)
enum { kRowMajor = 101, kColMajor = 102 };
enum { kNoTrans = 111, kTrans = 112, kConjTrans = 113 };
enum { kUpper = 121, kLower = 122 };
enum { kNonUnit = 131, kUnit = 132 };
enum { kLeft = 141, kRight = 142 };

constexpr int kNumSMs = 152;        // GB300: 2 dies x 76 SMs (queried at init)

// device status word bits (written by kernels, read by the host)
enum : unsigned {
  kErrMbarTimeout = 1u << 0,   // an mbarrier wait gave up
  kErrGridTimeout = 1u << 1,   // the grid barrier gave up
  kErrTmemAlloc   = 1u << 2,   // tcgen05.alloc could not be satisfied
};

// Host-side error handling: every CUDA runtime call of the library goes
// through ATLG_CHECK, which reports and aborts the calling entry point.
void fail(const char *what, cudaError_t e, const char *file, int line);
#define ATLG_CHECK(x)                                                     \
  do {                                                                    \
    cudaError_t e_ = (x);                                                 \
    if (e_ != cudaSuccess) ::atlg::fail(#x, e_, __FILE__, __LINE__);      \
  } while (0)

// ---------------------------------------------------------------- device
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Poll limit for mbarrier waits: ~2^26 try_wait rounds (each try_wait
// suspends for a hardware-chosen interval) is several seconds, far beyond
// any legitimate wait in these kernels.
constexpr unsigned kMbarPollLimit = 1u << 26;

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Spin (non-blocking tests, no suspension) bounded in time rather than in
// polls, for waits that end within microseconds in a correct run: false
// after `limit_ns` of global time.
__device__ __forceinline__ bool mbar_wait_for(uint64_t *bar, unsigned parity, unsigned long long limit_ns) {
  if (mbar_test_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_test_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
}

// Distributed shared memory: the address of the same variable in CTA `rank`
// of the cluster, and a 16-byte store into it that completes 16 bytes of the
// transaction count of an mbarrier in that CTA (the receiver waits on its
// own mbarrier; no cluster barrier and no fence on the sender).
__device__ __forceinline__ unsigned cluster_map(unsigned saddr, int rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_async16(unsigned raddr, uint4 v, unsigned rbar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(raddr),
      "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(rbar)
      : "memory");
}

// Bounded wait; returns false (and flags the status word) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned *status) {
  for (unsigned i = 0; i < kMbarPollLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if (status) atomicOr(status, kErrMbarTimeout);
  return false;
}

// TMA: 2-D tiled tensor load global -> shared, completion on an mbarrier.
// Coordinates are in elements, innermost first; out-of-range parts of the
// box are zero filled by the hardware.
__device__ __forceinline__ void tma_load_2d(void *smem_dst, const CUtensorMap *map, uint64_t *bar,
                                            int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}
// Start moving the 128-byte line holding p from memory into L2 (no register
// is written; the load that later reads the line finds it in L2).
__device__ __forceinline__ void prefetch_l2(const void *p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}
// x rounded to TF32 (10 mantissa bits), to nearest with ties away from zero:
// the high part of the 3xTF32 split (the low part is x minus it, exact).
__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// *p += v in L2 (round to nearest), no value returned: the issuing thread
// does not wait for it.
__device__ __forceinline__ void red_add_f64(double *p, double v) { (void)atomicAdd(p, v); }

// cp.async with zero fill: copies `src_bytes` (0 or the full size) and
// fills the rest of the destination with zeros.
__device__ __forceinline__ void cp_async8(void *smem_dst, const void *src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(smem_dst)),
               "l"(src), "r"(valid ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem_dst, const void *src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(smem_dst)),
               "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Grid-wide barrier for kernels whose CTAs are all co-resident (launched
// cooperatively).  `ctr` counts arrivals of the current generation; `gen`
// is bumped by the last arriver.  Waits are bounded.
constexpr unsigned kGridPollLimit = 1u << 25;
__device__ __forceinline__ bool grid_barrier(unsigned *ctr, volatile unsigned *gen, unsigned nblocks,
                                             unsigned *status) {
  __syncthreads();
  bool ok = true;
  if (threadIdx.x == 0) {
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(ctr, 1u) + 1u;
    if (arrived == nblocks) {
      *ctr = 0u;
      __threadfence();
      atomicAdd(const_cast<unsigned *>(gen), 1u);
    } else {
      unsigned i = 0;
      while (*gen == g) {
        if (++i > kGridPollLimit) {
          atomicOr(status, kErrGridTimeout);
          ok = false;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok;
}

// Grid-wide barrier on a monotonic arrival counter: barrier number t (from
// 1) of a grid of G co-resident CTAs completes when the counter reaches t*G.
// One atomic per CTA and polling of the same word; no reset, no second
// word.  Waits are bounded.
__device__ __forceinline__ bool grid_barrier_count(unsigned *ctr, unsigned target, unsigned *status) {
  __syncthreads();
  bool ok = true;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    volatile unsigned *vc = ctr;
    unsigned i = 0;
    while ((int)(*vc - target) < 0) {
      if (++i > kGridPollLimit) {
        atomicOr(status, kErrGridTimeout);
        ok = false;
        break;
      }
      if (i > 64) __nanosleep(20);
    }
    __threadfence();
  }
  __syncthreads();
  return ok;
}

// ---------------------------------------------------------------- host
struct Context;     // per-process library state (context.cuh)
Context &ctx();

// Encode a 2-D tiled tensor map over a column-major matrix:
// inner dimension `rows` (contiguous), outer `cols`, leading dimension `ld`
// (elements), box `box_rows` x `box_cols`.  Returns false when TMA cannot
// address the matrix (base not 16-byte aligned or ld*elem not a multiple of 16).
bool encode_tmap_2d(CUtensorMap *map, const void *base, CUtensorMapDataType dtype, int elem_bytes,
                    uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols,
                    CUtensorMapSwizzle swz = CU_TENSOR_MAP_SWIZZLE_NONE);

}  // namespace atlg
