// context.cuh -- per-process state shared by the C ABI and the drivers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace atlg {

// Device buffer slots reused across calls (grown on demand, never shrunk).
enum BufSlot {
  kBufA = 0, kBufB, kBufC, kBufPiv, kBufInfo, kBufW0, kBufW1, kBufW2, kBufW3, kBufW4, kBufW5,
  kNumSlots
};

struct Context {
  int device = 0;
  int num_sms = 152;
  int cc_major = 0, cc_minor = 0;
  cudaStream_t stream = nullptr;
  void *buf[kNumSlots] = {};
  size_t cap[kNumSlots] = {};
  void *buffer(int slot, size_t bytes);
};

}  // namespace atlg
