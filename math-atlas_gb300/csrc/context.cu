// context.cu -- per-process library state: the CUDA stream the host-pointer
// entry points run on, cached device buffers, the SM count and the
// tensor-map encoder (resolved from the driver at run time, so the library
// links only the CUDA runtime).
#include <mutex>
#include <stdlib.h>
#include <string.h>

#include "common.cuh"
#include "context.cuh"

namespace atlg {

void fail(const char *what, cudaError_t e, const char *file, int line) {
  fprintf(stderr, "atlas_gb300: CUDA error '%s' (%d) in %s at %s:%d\n", cudaGetErrorString(e), (int)e, what,
          file, line);
  fflush(stderr);
  abort();
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn g_encode = nullptr;

Context &ctx() {
  static Context *c = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    c = new Context();
    int dev = 0;
    ATLG_CHECK(cudaGetDevice(&dev));
    c->device = dev;
    cudaDeviceProp p;
    ATLG_CHECK(cudaGetDeviceProperties(&p, dev));
    c->num_sms = p.multiProcessorCount;
    c->cc_major = p.major;
    c->cc_minor = p.minor;
    int lo = 0, hi = 0;
    ATLG_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    // the library's own stream carries the factorization's critical path
    ATLG_CHECK(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, hi));
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    ATLG_CHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q == cudaDriverEntryPointSuccess) g_encode = reinterpret_cast<EncodeTiledFn>(fn);
  });
  return *c;
}

cudaStream_t stream_of(void *s) { return s ? static_cast<cudaStream_t>(s) : ctx().stream; }

void *Context::buffer(int slot, size_t bytes) {
  if (slot < 0 || slot >= kNumSlots) abort();
  if (bytes == 0) bytes = 16;
  if (cap[slot] < bytes) {
    if (buf[slot]) ATLG_CHECK(cudaFree(buf[slot]));
    buf[slot] = nullptr;
    cap[slot] = 0;
    size_t want = bytes + bytes / 8;   // grow with headroom
    want = (want + 255) & ~size_t(255);
    ATLG_CHECK(cudaMalloc(&buf[slot], want));
    cap[slot] = want;
  }
  return buf[slot];
}

cudaEvent_t Context::event() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  ATLG_CHECK(cudaEventCreate(&e));
  return e;
}

cudaStream_t Context::side_stream() {
  if (!side) {
    int lo = 0, hi = 0;
    ATLG_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    ATLG_CHECK(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, lo));   // lo = least urgent
  }
  return side;
}

cudaStream_t Context::outer_stream() {
  if (!outer) {
    int lo = 0, hi = 0;
    ATLG_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    ATLG_CHECK(cudaStreamCreateWithPriority(&outer, cudaStreamNonBlocking, lo));
  }
  return outer;
}

cudaEvent_t Context::sync_event(int i) {
  if (!sync_ev[i]) ATLG_CHECK(cudaEventCreateWithFlags(&sync_ev[i], cudaEventDisableTiming));
  return sync_ev[i];
}

bool encode_tmap_2d(CUtensorMap *map, const void *base, CUtensorMapDataType dtype, int elem_bytes,
                    uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols,
                    CUtensorMapSwizzle swz) {
  ctx();
  if (!g_encode) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
  if (((ld * (uint64_t)elem_bytes) & 15) != 0) return false;
  if (rows == 0 || cols == 0 || ld < rows) return false;
  if (((uint64_t)box_rows * elem_bytes) % 16 != 0) return false;
  cuuint64_t dims[2] = {rows, cols};
  cuuint64_t strides[1] = {ld * (uint64_t)elem_bytes};
  cuuint32_t box[2] = {box_rows, box_cols};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, dtype, 2, const_cast<void *>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace atlg
