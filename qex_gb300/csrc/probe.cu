// FMA-throughput probe: eight independent FMA chains per thread, 8 CTAs of
// 256 threads per SM, timed with CUDA events.
#include <cuda_runtime.h>

#include "qex_ks1d.h"
#include "qex_probe.h"

namespace {

constexpr int kThreads = 256;
constexpr int kCtasPerSm = 8;
constexpr int kMaxSms = 1024;

template <typename T>
__global__ void __launch_bounds__(kThreads) fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b;
    x1 = x1 * a + b;
    x2 = x2 * a + b;
    x3 = x3 * a + b;
    x4 = x4 * a + b;
    x5 = x5 * a + b;
    x6 = x6 * a + b;
    x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double time_tflops(T* buf, int blocks, int iters, cudaStream_t s) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, kThreads, 0, s>>>(buf, iters / 8, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0, s);
  fma_chains<T><<<blocks, kThreads, 0, s>>>(buf, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * kThreads;
  return ms > 0.0f ? flops / (ms * 1e-3) / 1e12 : 0.0;
}

}  // namespace

extern "C" {

size_t qex_probe_workspace_size(void) {
  return sizeof(double) * (size_t)kMaxSms * kCtasPerSm * kThreads;
}

int qex_probe_fma_peak(double* fp64_tflops, double* fp32_tflops, void* workspace,
                       size_t workspace_bytes, void* stream) {
  if (!fp64_tflops || !fp32_tflops || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_probe_workspace_size()) return QEX_BAD_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1 || sms > kMaxSms) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = sms * kCtasPerSm;
  *fp64_tflops = time_tflops<double>(static_cast<double*>(workspace), blocks, 2048, s);
  *fp32_tflops = time_tflops<float>(static_cast<float*>(workspace), blocks, 65536, s);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
