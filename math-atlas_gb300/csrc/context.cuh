// context.cuh -- per-process state shared by the C ABI and the drivers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <vector>

namespace atlg {

// Device buffer slots reused across calls (grown on demand, never shrunk).
enum BufSlot {
  kBufA = 0, kBufB, kBufC, kBufPiv, kBufInfo, kBufW0, kBufW1, kBufW2, kBufW3, kBufW4, kBufW5, kBufW6, kBufW7, kBufS0, kBufS1, kBufS2, kBufT0, kBufT1, kBufV0, kBufV1, kBufChol, kBufTrmm, kBufX0, kBufX1, kBufX2, kBufS3, kBufS4, kBufS5, kBufTri, kBufV2, kBufIamax, kBufTrsvL, kBufTrsvU, kBufGemv, kBufTrsmInv, kBufT2, kBufRowPart, kBufFlag,
  kNumSlots
};

// Launch accounting and per-kernel timing used by the benchmark: every kernel
// launch of the library bumps `launches`; when `prof` is on, the GEMM driver
// brackets each launch with CUDA events on its stream.
struct ProfRec {
  cudaEvent_t beg, end;
  double flops;
};

struct Context {
  int device = 0;
  int num_sms = 152;
  int cc_major = 0, cc_minor = 0;
  cudaStream_t stream = nullptr;
  void *buf[kNumSlots] = {};
  size_t cap[kNumSlots] = {};
  void *buffer(int slot, size_t bytes);
  unsigned long long launches = 0;
  bool prof = false;
  std::vector<ProfRec> recs;
  bool prof_panels = false;          // LU panels: events before and after each panel launch
  std::vector<ProfRec> panel_recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t event();
  cudaStream_t side = nullptr;       // low-priority stream for overlapped updates
  cudaStream_t outer = nullptr;      // a second one, for a driver whose inner steps use `side`
  cudaEvent_t sync_ev[6] = {};       // cross-stream ordering (no timing)
  cudaStream_t side_stream();
  cudaStream_t outer_stream();
  cudaEvent_t sync_event(int i);
};

inline void note_launch(unsigned n = 1);

Context &ctx();
// the stream an atlg_*_dev call runs on: the caller's, or for NULL the
// library's own non-blocking stream
cudaStream_t stream_of(void *s);
inline void note_launch(unsigned n) { ctx().launches += n; }

}  // namespace atlg
