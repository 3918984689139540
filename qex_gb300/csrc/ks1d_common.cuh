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
constexpr int kPhases = 16;  // phase timers per molecule
// Warm route when |dv_KS| < kFastGap * (smallest gap): below 1/2 the Weyl
// intervals of neighbouring eigenvalues are disjoint, which the check needs.
constexpr double kFastGap = 0.45;
constexpr int kChunk = 32;   // points per chunk of the streamed FP32 solves (default)
constexpr int kMaxChunk = 64;  // the largest chunk (qex_ks1d_options.solve_chunk: 16, 32, 64)
constexpr int kRing = 4;     // chunks in the shared-memory ring (kRing - 1 in flight)
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
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ float warp_minf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Two warp sums for the FP64 additions of one: after the first exchange the
// lower half-warp carries a, the upper half b.  FP64 operations issue at a
// small fraction of the FP32 rate, so the saving is in pipe time, not latency.
__device__ __forceinline__ void warp_sum2(double& a, double& b, int lane) {
  const bool hi = (lane & 16) != 0;
  double v = hi ? b : a;
  v += __shfl_xor_sync(kFull, hi ? a : b, 16);
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  a = __shfl_sync(kFull, v, 0);
  b = __shfl_sync(kFull, v, 16);
}

// Asynchronous global -> shared copies (sm_80+ cp.async); the caller commits
// and waits on groups.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int kPending>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(kPending) : "memory");
}

// FP64 reciprocal, quotient and inverse square root by Newton's iteration
// from an FP32 seed: each step squares the relative error (about 2^-22 ->
// 2^-44 -> below FP64 rounding).  For |x| within the FP32 normal range, which
// the callers guarantee (norms and Rayleigh quotients of O(1) vectors).
__device__ __forceinline__ double recip_nr(double x) {
  double r = (double)__fdividef(1.0f, (float)x);
  r = fma(r, fma(-x, r, 1.0), r);
  return fma(r, fma(-x, r, 1.0), r);
}
__device__ __forceinline__ double div_nr(double a, double b) {
  const double r = recip_nr(b);
  const double q = a * r;
  return fma(r, fma(-b, q, a), q);
}
__device__ __forceinline__ double rsqrt_nr(double x) {
  double y = (double)rsqrtf((float)x);
  const double h = 0.5 * x;
  y = y * fma(-h * y, y, 1.5);
  return y * fma(-h * y, y, 1.5);
}

}  // namespace qex
