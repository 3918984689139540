// Shared device helpers for the 1D Kohn-Sham kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "qex_ks1d.h"

namespace qex {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarp = 32;
constexpr int kMaxEig = QEX_KS1D_MAX_EIGENPAIRS;  // eigenpairs computed per molecule
constexpr int kMaxBis = kMaxEig + 1;              // eigenvalues bracketed (one extra)
constexpr int kShiftsPerLane = 4;                 // Sturm shifts evaluated per lane per pass
constexpr int kSamples = kWarp * kShiftsPerLane;
constexpr int kMaxPasses = 48;
constexpr int kMaxRefineSteps = 10;
constexpr int kPad64 = 2;   // zero padding either side of the FP64 staging vector
constexpr int kPadMlp = 8;  // half window

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

}  // namespace qex
