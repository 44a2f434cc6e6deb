// Device scratch of the tensor-core GEMMs, owned by the calling host thread, one set per device.
//
// The library's threading model is one host thread per context, contexts independent: a buffer
// shared by the whole process would let two contexts on two threads (or two devices) overwrite each
// other's packed operands. A set per (thread, device) is reused only by the next call of the same
// thread on the same device, which is stream-ordered after the previous one because every API call
// synchronises its stream before returning. Growing a buffer waits for the device first. The buffers
// are released when the thread exits.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace dg {

struct ScratchBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// Buffers of one device: up to four growable arrays, an error word, a one-time-init flag.
struct DeviceScratch {
  ScratchBuf buf[4];
  int *err = nullptr;
  bool attr = false;
};

class ThreadScratch {
 public:
  // The current device's set (created on first use).
  DeviceScratch &current() {
    int d = 0;
    cudaGetDevice(&d);
    if ((int)dev_.size() <= d) dev_.resize(d + 1);
    return dev_[d];
  }
  ~ThreadScratch() {
    for (size_t d = 0; d < dev_.size(); ++d) {
      bool any = dev_[d].err != nullptr;
      for (const ScratchBuf &b : dev_[d].buf) any = any || b.p != nullptr;
      if (!any || cudaSetDevice((int)d) != cudaSuccess) continue;
      for (ScratchBuf &b : dev_[d].buf)
        if (b.p) cudaFree(b.p);
      if (dev_[d].err) cudaFree(dev_[d].err);
    }
  }

 private:
  std::vector<DeviceScratch> dev_;
};

// Grow b to at least `bytes` (contents are not kept). Returns a cudaError_t value.
inline int scratch_reserve(ScratchBuf &b, size_t bytes) {
  if (bytes <= b.bytes) return 0;
  cudaDeviceSynchronize();
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  const cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    cudaGetLastError();   // an out-of-memory here is reported by the return value only
    return (int)e;
  }
  b.bytes = bytes;
  return 0;
}

// The error word of the set (allocated and cleared on first use). Returns a cudaError_t value.
inline int scratch_err(DeviceScratch &d) {
  if (d.err) return 0;
  const cudaError_t e = cudaMalloc((void **)&d.err, sizeof(int));
  if (e != cudaSuccess) {
    d.err = nullptr;
    cudaGetLastError();
    return (int)e;
  }
  return (int)cudaMemset(d.err, 0, sizeof(int));
}

// Read and clear the error word of the current device's set.
inline int scratch_take_err(DeviceScratch &d) {
  if (!d.err) return 0;
  int h = 0;
  cudaMemcpy(&h, d.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (h) cudaMemset(d.err, 0, sizeof(int));
  return h;
}

}  // namespace dg
