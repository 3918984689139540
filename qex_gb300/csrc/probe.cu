// Throughput probes: eight independent FMA chains per thread (FP64 and FP32
// CUDA cores), and FP64 tensor-core MMA chains, 8 CTAs of 256 threads per SM,
// timed with CUDA events.
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

// FP64 tensor-core (DMMA) throughput: four independent accumulator chains of
// mma.sync per warp, operands held in registers (no memory traffic).
template <int kShape>  // 0: m8n8k4, 1: m16n8k16
__global__ void __launch_bounds__(kThreads) dmma_chains(double* out, int iters) {
  const double base = threadIdx.x * 1e-3;
  if (kShape == 0) {
    double c[4][2] = {};
    const double a = base, b = 0.5;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(c[q][0]), "+d"(c[q][1])
                     : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  } else {
    double c[4][4] = {};
    double a[8], b[4];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = base + i;
#pragma unroll
    for (int i = 0; i < 4; ++i) b[i] = 0.5 + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
            "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
            : "+d"(c[q][0]), "+d"(c[q][1]), "+d"(c[q][2]), "+d"(c[q][3])
            : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]),
              "d"(a[7]), "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  }
}

template <int kShape>
double time_dmma(double* buf, int blocks, int iters, cudaStream_t s) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dmma_chains<kShape><<<blocks, kThreads, 0, s>>>(buf, iters / 8);  // warm-up
  cudaEventRecord(e0, s);
  dmma_chains<kShape><<<blocks, kThreads, 0, s>>>(buf, iters);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double per_mma = kShape == 0 ? 2.0 * 8 * 8 * 4 : 2.0 * 16 * 8 * 16;
  const double warps = (double)blocks * kThreads / 32.0;
  const double flops = per_mma * 4.0 * iters * warps;
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

int qex_probe_dmma_peak(double* m8n8k4_tflops, double* m16n8k16_tflops, void* workspace,
                        size_t workspace_bytes, void* stream) {
  if (!m8n8k4_tflops || !m16n8k16_tflops || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_probe_workspace_size()) return QEX_BAD_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1 || sms > kMaxSms) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = sms * kCtasPerSm;
  *m8n8k4_tflops = time_dmma<0>(static_cast<double*>(workspace), blocks, 1024, s);
  *m16n8k16_tflops = time_dmma<1>(static_cast<double*>(workspace), blocks, 256, s);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
