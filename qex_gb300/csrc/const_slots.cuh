// Host-side staging of per-launch network weights into __constant__ slots.
//
// A kernel that reads its weights from constant memory gets every weight as a
// warp-uniform operand of the FMA that uses it; loaded per lane from global or
// shared memory, each weight is written into 32 registers, and that register
// write-back bounds the small per-point networks of the 1D kernels.
//
// A slot belongs to the stream that last used it; launches on that stream
// re-stage it in stream order.  A slot that changes hands is first waited on
// (the previous owner's last launch), so concurrent launches on different
// streams with different weights never share a slot while one of them runs.
// Staging is refused under stream capture: a graph that replays a slot's copy
// and launch later would hold the slot outside this table's ownership rules,
// and another stream given the slot meanwhile could overwrite the weights
// while the graph runs.  Callers return QEX_BAD_ARG for a launch attempted
// under capture (capturing_refused()).
//
// Internal linkage throughout: each translation unit has its own constant
// arrays, and the staging code must write the array its kernels read.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

namespace qex {
namespace {

constexpr int kConstMaxDevices = 64;

template <int kSlots>
struct ConstSlots {
  struct Table {
    cudaStream_t owner[kSlots];
    cudaEvent_t done[kSlots];
    bool used[kSlots];
    int next;
  };
  std::mutex mu;
  Table tab[kConstMaxDevices];
};

template <int kSlots>
class ConstStage {
 public:
  // Copies `bytes` from `src` (kind: device or host source) into a slot of the
  // constant array `symbol` (kSlots slots of `slot_bytes`) for a launch on `stream`.
  ConstStage(ConstSlots<kSlots>& slots, const void* symbol, size_t slot_bytes, const void* src,
             size_t bytes, cudaMemcpyKind kind, cudaStream_t stream)
      : slots_(slots), lock_(slots.mu), stream_(stream) {
    if (bytes > slot_bytes || cudaGetDevice(&dev_) != cudaSuccess || dev_ < 0 ||
        dev_ >= kConstMaxDevices)
      return;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) return;
    if (cap != cudaStreamCaptureStatusNone) {
      capturing_ = true;
      return;
    }
    auto& t = slots.tab[dev_];
    int s = -1;
    for (int i = 0; i < kSlots; ++i)
      if (t.used[i] && t.owner[i] == stream) s = i;
    if (s < 0) {
      s = t.next;
      t.next = (t.next + 1) % kSlots;
      if (!t.used[s]) {
        if (cudaEventCreateWithFlags(&t.done[s], cudaEventDisableTiming) != cudaSuccess) return;
        t.used[s] = true;
      } else if (cudaStreamWaitEvent(stream, t.done[s], 0) != cudaSuccess) {
        return;
      }
      t.owner[s] = stream;
    }
    if (cudaMemcpyToSymbolAsync(symbol, src, bytes, slot_bytes * (size_t)s, kind, stream) !=
        cudaSuccess)
      return;
    slot_ = s;
  }
  int slot() const { return slot_; }
  // True when the stream was capturing: nothing was staged.
  bool capturing_refused() const { return capturing_; }
  // Call after the launch that reads the slot.
  bool finish() {
    if (slot_ < 0) return false;
    return cudaEventRecord(slots_.tab[dev_].done[slot_], stream_) == cudaSuccess;
  }

 private:
  ConstSlots<kSlots>& slots_;
  std::lock_guard<std::mutex> lock_;
  cudaStream_t stream_;
  int dev_ = -1;
  int slot_ = -1;
  bool capturing_ = false;
};

}  // namespace
}  // namespace qex
