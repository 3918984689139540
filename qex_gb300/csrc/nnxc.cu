// Neural XC functional on the 3D grid (FP32 network, FP64 interface).
//
// Reference: qedft/train/td/xc.py:12-47 (get_exc_and_vrho: exc = network(rho),
// vrho = vjp of the network with ones) with the local MLP of
// qedft/train/td/trainer_legacy_no_jit.py:56-62 (per-point input) and :98-107
// (features [H, H, 1], gelu hidden activations, output -scale * swish):
//   z1 = rho w1 + b1,  h1 = gelu(z1)           (1 -> H, rank one)
//   z2 = h1 W2 + b2,   h2 = gelu(z2)           (H -> H, the GEMM)
//   z3 = h2 . w3 + b3, exc = -scale swish(z3)
//   vrho = d exc / d rho (the chain rule back through the same layers).
// Two FP32 SIMT GEMMs over 64-point x 64-unit tiles: the forward one builds h1
// while staging its A tile and reduces h2 . w3 in its epilogue; the backward
// one builds dz2 = dz3 w3 gelu'(z2) while staging and reduces dh1 gelu'(z1) w1
// in its epilogue.  Per-tile partial sums are added in a fixed order
// (deterministic).  gelu is the tanh form (flax's default).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kBM = 64;   // points per tile
constexpr int kBN = 64;   // hidden units per tile
constexpr int kBK = 16;   // k-step
constexpr int kNT = 256;  // 16 x 16 threads, 4 x 4 outputs each
constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float gelu_f(float x, float& d) {
  const float x2 = x * x;
  const float u = kGeluC * fmaf(kGeluA * x2, x, x);
  const float t = tanhf(u);
  d = fmaf(0.5f * x * (1.0f - t * t) * kGeluC, fmaf(3.0f * kGeluA, x2, 1.0f), 0.5f * (1.0f + t));
  return 0.5f * x * (1.0f + t);
}

struct NetView {
  const float* w1;  // H
  const float* b1;  // H
  const float* W2;  // H x H, row = input unit
  const float* b2;  // H
  const float* w3;  // H
  const float* b3;  // 1
};

__device__ __forceinline__ NetView net_view(const float* p, int H) {
  NetView v;
  v.w1 = p;
  v.b1 = p + H;
  v.W2 = p + 2 * H;
  v.b2 = p + 2 * H + (size_t)H * H;
  v.w3 = v.b2 + H;
  v.b3 = v.w3 + H;
  return v;
}

// Forward: z2 = gelu(rho w1 + b1) W2 + b2 stored to Z2 (G x H); part1[tn][g] =
// sum over the tile's units of gelu(z2) w3.
__global__ void __launch_bounds__(kNT) nn_forward_kernel(long long G, int H, const double* rho,
                                                         const float* params, float* Z2,
                                                         float* part1) {
  const NetView net = net_view(params, H);
  __shared__ float As[kBK][kBM + 1];
  __shared__ float Bs[kBK][kBN + 1];
  __shared__ float red[kBM][17];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long long g0 = (long long)blockIdx.x * kBM;
  const int n0 = blockIdx.y * kBN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < H; k0 += kBK) {
    for (int e = threadIdx.x; e < kBK * kBM; e += kNT) {
      const int k = e % kBK, r = e / kBK;  // adjacent threads: adjacent units
      const long long g = g0 + r;
      float h = 0.0f;
      if (g < G && k0 + k < H) {
        float d;
        h = gelu_f(fmaf((float)rho[g], net.w1[k0 + k], net.b1[k0 + k]), d);
      }
      As[k][r] = h;
    }
    for (int e = threadIdx.x; e < kBK * kBN; e += kNT) {
      const int k = e / kBN, c = e % kBN;
      Bs[k][c] = (k0 + k < H && n0 + c < H) ? net.W2[(size_t)(k0 + k) * H + n0 + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[k][ty * 4 + q];
        b[q] = Bs[k][tx * 4 + q];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ty * 4 + i;
    const long long g = g0 + r;
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx * 4 + j;
      if (g < G && c < H) {
        const float z = acc[i][j] + net.b2[c];
        Z2[(size_t)g * H + c] = z;
        float d;
        s = fmaf(gelu_f(z, d), net.w3[c], s);
      }
    }
    red[r][tx] = s;
  }
  __syncthreads();
  if (threadIdx.x < kBM) {
    const long long g = g0 + threadIdx.x;
    float s = 0.0f;
    for (int t = 0; t < 16; ++t) s += red[threadIdx.x][t];
    if (g < G) part1[(size_t)blockIdx.y * G + g] = s;
  }
}

// exc and dexc/dz3 per point; with weights, per-block partials of
// (sum w rho, sum w rho exc) in FP64 (256 threads).
__global__ void __launch_bounds__(256) nn_output_kernel(long long G, int H, int ntiles,
                                                        const float* params, const float* part1,
                                                        float scale, const double* rho,
                                                        const double* w, double* exc, float* dz3,
                                                        double* sums_part) {
  const NetView net = net_view(params, H);
  double ne = 0.0, ex = 0.0;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (long long)gridDim.x * blockDim.x) {
    float z = net.b3[0];
    for (int t = 0; t < ntiles; ++t) z += part1[(size_t)t * G + g];
    const float sg = 1.0f / (1.0f + expf(-z));
    const double e = (double)(-scale * z * sg);
    exc[g] = e;
    dz3[g] = -scale * sg * fmaf(z, 1.0f - sg, 1.0f);
    if (w) {
      const double a = w[g] * rho[g];
      ne += a;
      ex = fma(a, e, ex);
    }
  }
  if (!w) return;
  __shared__ double red[2][8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
    ex += __shfl_xor_sync(0xffffffffu, ex, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = ne;
    red[1][threadIdx.x >> 5] = ex;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < 8; ++i) {
      a += red[0][i];
      b += red[1][i];
    }
    sums_part[2 * blockIdx.x] = a;
    sums_part[2 * blockIdx.x + 1] = b;
  }
}

__global__ void nn_sums_kernel(int nblocks, const double* part, double* sums) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nblocks; ++i) {
      a += part[2 * i];
      b += part[2 * i + 1];
    }
    sums[0] = a;
    sums[1] = b;
  }
}

// Backward: dh1 = (dz3 w3 o gelu'(z2)) W2^T; part2[tk][g] = sum over the
// tile's units k of dh1 gelu'(z1) w1.
__global__ void __launch_bounds__(kNT) nn_backward_kernel(long long G, int H, const double* rho,
                                                          const float* params, const float* Z2,
                                                          const float* dz3, float* part2) {
  const NetView net = net_view(params, H);
  __shared__ float As[kBK][kBM + 1];
  __shared__ float Bs[kBK][kBN + 1];
  __shared__ float red[kBM][17];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long long g0 = (long long)blockIdx.x * kBM;
  const int m0 = blockIdx.y * kBN;  // output units (rows of W2)
  float acc[4][4] = {};
  for (int n0 = 0; n0 < H; n0 += kBK) {
    for (int e = threadIdx.x; e < kBK * kBM; e += kNT) {
      const int k = e % kBK, r = e / kBK;  // adjacent threads: adjacent units of Z2
      const long long g = g0 + r;
      float v = 0.0f;
      if (g < G && n0 + k < H) {
        float d;
        gelu_f(Z2[(size_t)g * H + n0 + k], d);
        v = dz3[g] * net.w3[n0 + k] * d;
      }
      As[k][r] = v;
    }
    for (int e = threadIdx.x; e < kBK * kBN; e += kNT) {
      const int k = e % kBK, c = e / kBK;  // adjacent threads: adjacent columns of W2
      // B[k][c] = W2^T[n0 + k][m0 + c] = W2[m0 + c][n0 + k]
      Bs[k][c] = (n0 + k < H && m0 + c < H) ? net.W2[(size_t)(m0 + c) * H + n0 + k] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[k][ty * 4 + q];
        b[q] = Bs[k][tx * 4 + q];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ty * 4 + i;
    const long long g = g0 + r;
    float s = 0.0f;
    if (g < G) {
      const float x = (float)rho[g];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = m0 + tx * 4 + j;
        if (c < H) {
          float d;
          gelu_f(fmaf(x, net.w1[c], net.b1[c]), d);
          s = fmaf(acc[i][j] * d, net.w1[c], s);
        }
      }
    }
    red[r][tx] = s;
  }
  __syncthreads();
  if (threadIdx.x < kBM) {
    const long long g = g0 + threadIdx.x;
    float s = 0.0f;
    for (int t = 0; t < 16; ++t) s += red[threadIdx.x][t];
    if (g < G) part2[(size_t)blockIdx.y * G + g] = s;
  }
}

__global__ void nn_vrho_kernel(long long G, int ntiles, const float* part2, double* vrho) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (long long)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int t = 0; t < ntiles; ++t) s += part2[(size_t)t * G + g];
    vrho[g] = (double)s;
  }
}

}  // namespace

extern "C" {

constexpr int kMaxOutBlocks = 4096;

size_t qex_td_nn_xc_workspace_size(int64_t num_points, int32_t hidden) {
  if (num_points < 0 || hidden < 1) return 0;
  const size_t tiles = (size_t)(hidden + kBN - 1) / kBN;
  // FP64 block partials of the sums, then FP32 Z2 (G x H), dz3 (G) and two
  // per-tile partial planes (tiles x G)
  return sizeof(double) * 2 * kMaxOutBlocks +
         sizeof(float) * (size_t)num_points * ((size_t)hidden + 1 + 2 * tiles) + 256;
}

int qex_td_nn_xc(int64_t num_points, int32_t hidden, const double* rho, const double* weights,
                 const float* params, double scale, double* exc, double* vrho, double* sums,
                 void* workspace, size_t workspace_bytes, void* stream) {
  if (num_points < 0 || hidden < 1) return QEX_BAD_ARG;
  if (num_points == 0) return QEX_OK;
  if (!rho || !params || !exc || !vrho || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_nn_xc_workspace_size(num_points, hidden)) return QEX_BAD_ARG;
  const long long G = num_points;
  const int tiles = (hidden + kBN - 1) / kBN;
  const long long gt = (G + kBM - 1) / kBM;
  if (gt > 0x7fffffffLL || tiles > 65535) return QEX_BAD_ARG;
  if ((weights == nullptr) != (sums == nullptr)) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* sums_part = static_cast<double*>(workspace);
  float* Z2 = reinterpret_cast<float*>(sums_part + 2 * kMaxOutBlocks);
  float* dz3 = Z2 + (size_t)G * hidden;
  float* part1 = dz3 + G;
  float* part2 = part1 + (size_t)tiles * G;
  const dim3 grid((unsigned)gt, (unsigned)tiles);
  nn_forward_kernel<<<grid, kNT, 0, s>>>(G, hidden, rho, params, Z2, part1);
  const int eb = (int)((G + 255) / 256 < kMaxOutBlocks ? (G + 255) / 256 : kMaxOutBlocks);
  nn_output_kernel<<<eb, 256, 0, s>>>(G, hidden, tiles, params, part1, (float)scale, rho, weights,
                                      exc, dz3, sums_part);
  if (weights) nn_sums_kernel<<<1, 32, 0, s>>>(eb, sums_part, sums);
  nn_backward_kernel<<<grid, kNT, 0, s>>>(G, hidden, rho, params, Z2, dz3, part2);
  nn_vrho_kernel<<<eb, 256, 0, s>>>(G, tiles, part2, vrho);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Global network (qedft/train/td/trainer_legacy_no_jit.py:46-53 with the MLP of
// :98-107, consumed as the "NN-AmplitudeEncoding" xctype of
// qedft/train/td/numint_legacy.py:311-333): the whole density vector is one
// input, exc = sum network(rho) is a scalar and vrho = d exc / d rho (G).
// Layer 1 is a G x H GEMV (W1 row-major (G, H)), so the first and last kernels
// stream W1 from memory coalesced; the H-wide middle runs in one CTA.
// ---------------------------------------------------------------------------
namespace {

constexpr int kGChunk = 128;   // grid points per z1 partial
constexpr int kGlobThreads = 256;
constexpr int kMaxHidden = 1024;

struct GlobView {
  const float* W1;  // G x H
  const float* b1;
  const float* W2;  // H x H
  const float* b2;
  const float* w3;
  const float* b3;
};

__device__ __forceinline__ GlobView glob_view(const float* p, long long G, int H) {
  GlobView v;
  v.W1 = p;
  v.b1 = p + (size_t)G * H;
  v.W2 = v.b1 + H;
  v.b2 = v.W2 + (size_t)H * H;
  v.w3 = v.b2 + H;
  v.b3 = v.w3 + H;
  return v;
}

// part[c][h] = sum over chunk c of rho_g W1[g][h]
__global__ void __launch_bounds__(kGlobThreads) glob_z1_kernel(long long G, int H,
                                                               const double* rho,
                                                               const float* params, float* part) {
  const GlobView net = glob_view(params, G, H);
  const int h = blockIdx.y * kGlobThreads + threadIdx.x;
  const long long g0 = (long long)blockIdx.x * kGChunk;
  if (h >= H) return;
  float acc = 0.0f;
  const long long g1 = min(G, g0 + kGChunk);
  for (long long g = g0; g < g1; ++g) acc = fmaf((float)rho[g], net.W1[(size_t)g * H + h], acc);
  part[(size_t)blockIdx.x * H + h] = acc;
}

// One CTA: z1, h1 = gelu, z2, h2, z3, out and the backward to dz1 (global),
// exc sum into sums[1].
__global__ void __launch_bounds__(kMaxHidden) glob_mid_kernel(long long G, int H, int nchunks,
                                                              const float* params,
                                                              const float* part, float scale,
                                                              float* dz1, double* sums) {
  const GlobView net = glob_view(params, G, H);
  __shared__ float h1[kMaxHidden], d1[kMaxHidden], dz2[kMaxHidden];
  __shared__ float red[32];
  const int h = threadIdx.x;
  if (h < H) {
    float z = net.b1[h];
    for (int c = 0; c < nchunks; ++c) z += part[(size_t)c * H + h];
    float d;
    h1[h] = gelu_f(z, d);
    d1[h] = d;
  }
  __syncthreads();
  float d2 = 0.0f, contrib = 0.0f;
  if (h < H) {
    float z = net.b2[h];
    for (int k = 0; k < H; ++k) z = fmaf(h1[k], net.W2[(size_t)k * H + h], z);
    const float a = gelu_f(z, d2);
    contrib = a * net.w3[h];
  }
  // z3 = sum_h h2 w3 + b3 (fixed-order block reduction)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
  if ((h & 31) == 0) red[h >> 5] = contrib;
  __syncthreads();
  float z3 = net.b3[0];
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) z3 += red[i];
  const float sg = 1.0f / (1.0f + expf(-z3));
  const float dz3 = -scale * sg * fmaf(z3, 1.0f - sg, 1.0f);
  if (h < H) dz2[h] = dz3 * net.w3[h] * d2;
  __syncthreads();
  if (h < H) {
    float s = 0.0f;
    for (int j = 0; j < H; ++j) s = fmaf(net.W2[(size_t)h * H + j], dz2[j], s);
    dz1[h] = s * d1[h];
  }
  if (h == 0) sums[1] = (double)(-scale * z3 * sg);
}

// vrho[g] = sum_h W1[g][h] dz1[h] (one warp per grid point); sums[0] partials.
__global__ void __launch_bounds__(kGlobThreads) glob_vrho_kernel(long long G, int H,
                                                                 const double* rho,
                                                                 const double* w,
                                                                 const float* params,
                                                                 const float* dz1, double* vrho,
                                                                 double* ne_part) {
  const GlobView net = glob_view(params, G, H);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int wpb = kGlobThreads / 32;
  double ne = 0.0;
  for (long long g = (long long)blockIdx.x * wpb + wid; g < G; g += (long long)gridDim.x * wpb) {
    float s = 0.0f;
    for (int h = lane; h < H; h += 32) s = fmaf(net.W1[(size_t)g * H + h], dz1[h], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      vrho[g] = (double)s;
      if (w) ne += w[g] * rho[g];
    }
  }
  __shared__ double red[kGlobThreads / 32];
  if (lane == 0) red[wid] = ne;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int i = 0; i < wpb; ++i) a += red[i];
    ne_part[blockIdx.x] = a;
  }
}

__global__ void glob_sum_kernel(int nblocks, const double* part, double* sums) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0;
    for (int i = 0; i < nblocks; ++i) a += part[i];
    sums[0] = a;
  }
}

constexpr int kGlobVrhoBlocks = 1024;

}  // namespace

extern "C" {

size_t qex_td_nn_xc_global_workspace_size(int64_t num_points, int32_t hidden) {
  if (num_points < 1 || hidden < 1 || hidden > kMaxHidden) return 0;
  const size_t chunks = (size_t)((num_points + kGChunk - 1) / kGChunk);
  return sizeof(float) * (chunks * (size_t)hidden + (size_t)hidden) +
         sizeof(double) * kGlobVrhoBlocks + 256;
}

int qex_td_nn_xc_global(int64_t num_points, int32_t hidden, const double* rho,
                        const double* weights, const float* params, double scale, double* vrho,
                        double* sums, void* workspace, size_t workspace_bytes, void* stream) {
  if (num_points < 1 || hidden < 1 || hidden > kMaxHidden) return QEX_BAD_ARG;
  if (!rho || !weights || !params || !vrho || !sums || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_nn_xc_global_workspace_size(num_points, hidden)) return QEX_BAD_ARG;
  const long long G = num_points;
  const int chunks = (int)((G + kGChunk - 1) / kGChunk);
  if (chunks > 0x7fffffff) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* ne_part = static_cast<double*>(workspace);
  float* part = reinterpret_cast<float*>(ne_part + kGlobVrhoBlocks);
  float* dz1 = part + (size_t)chunks * hidden;
  glob_z1_kernel<<<dim3((unsigned)chunks, (hidden + kGlobThreads - 1) / kGlobThreads), kGlobThreads,
                   0, s>>>(G, hidden, rho, params, part);
  const int mt = ((hidden + 31) / 32) * 32;
  glob_mid_kernel<<<1, mt, 0, s>>>(G, hidden, chunks, params, part, (float)scale, dz1, sums);
  const int vb = (int)((G + 7) / 8 < kGlobVrhoBlocks ? (G + 7) / 8 : kGlobVrhoBlocks);
  glob_vrho_kernel<<<vb, kGlobThreads, 0, s>>>(G, hidden, rho, weights, params, dz1, vrho, ne_part);
  glob_sum_kernel<<<1, 32, 0, s>>>(vb, ne_part, sums);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
