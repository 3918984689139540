// GGA pieces of the 3D numint, qedft/train/td/numint_legacy.py:175-198 (the
// GGA branch of nr_rks): AO values with first derivatives (ao_deriv = 1),
// rho and its gradient (make_rho "GGA"), the GGA potential matrix
// V = ao0^T sum_n wv_n ao_n + transpose (_rks_gga_wv0, _scale_ao, _dot_ao_ao),
// and one GGA functional restated from its publication, PBE exchange
// (Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)); libxc is not available.
//
// Layouts: ao4 is (4, G, nao): values, then d/dx, d/dy, d/dz (pyscf's
// ao_deriv = 1 order); rho4 is (4, G): rho, drho/dx, /dy, /dz; wv is (4, G).
// All FP64; the products are 64 x 64-tiled like the LDA kernels in td.cu and
// split over grid chunks so that they span the GPU; partial results are summed
// in a fixed order (deterministic).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cart.cuh"
#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kThreads = 256;
constexpr int kTile = 64;
constexpr int kTileK = 16;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kCtas = 304;  // target CTAs of one potential-matrix product (2 per SM)

int grid_for(long long work, int threads) {
  long long g = (work + threads - 1) / threads;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// AO values and gradients
// ---------------------------------------------------------------------------
__global__ void eval_ao_d1_kernel(long long G, const double* __restrict__ coords, int ns,
                                  const double* __restrict__ centers, const int* __restrict__ l,
                                  const int* __restrict__ poff, const int* __restrict__ aooff,
                                  const double* __restrict__ ex, const double* __restrict__ co,
                                  int nao, double* __restrict__ ao) {
  const long long total = G * ns;
  const long long plane = G * nao;
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const long long g = it / ns;
    const int s = (int)(it - g * ns);
    const double d[3] = {coords[3 * g] - centers[3 * s], coords[3 * g + 1] - centers[3 * s + 1],
                         coords[3 * g + 2] - centers[3 * s + 2]};
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    // radial part and its derivative with respect to r2, times 2
    double rad = 0.0, drad = 0.0;
    for (int p = poff[s]; p < poff[s + 1]; ++p) {
      const double t = co[p] * exp(-ex[p] * r2);
      rad += t;
      drad -= 2.0 * ex[p] * t;
    }
    double* row = ao + g * nao + aooff[s];
    const int ls = l[s];
    if (ls < 0 || ls > kMaxShellL) continue;
    for (int k = 0; k < ncart(ls); ++k) {
      int c[3];
      cart_exponents(ls, k, c);
      const double px = cart_pow(d[0], c[0]), py = cart_pow(d[1], c[1]), pz = cart_pow(d[2], c[2]);
      const double m = px * py * pz;
      row[k] = m * rad;
      // d/dq (m rad) = (dm/dq) rad + m drad d_q
      const double dm[3] = {cart_dpow(d[0], c[0]) * py * pz, px * cart_dpow(d[1], c[1]) * pz,
                            px * py * cart_dpow(d[2], c[2])};
      for (int q = 0; q < 3; ++q) row[(q + 1) * plane + k] = dm[q] * rad + m * drad * d[q];
    }
  }
}

// ---------------------------------------------------------------------------
// rho4: T = ao0 D (64 x 64 tiles); the epilogue takes the row dots of T with
// the four AO components; partials per column tile, (4, tiles, G)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) rho_gga_kernel(long long G, int n,
                                                           const double* __restrict__ ao,
                                                           const double* __restrict__ D,
                                                           double* __restrict__ part) {
  __shared__ double As[kTileK][kTile + 1];
  __shared__ double Bs[kTileK][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long long row0 = (long long)blockIdx.x * kTile;
  const int col0 = blockIdx.y * kTile;
  const long long plane = G * n;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < n; k0 += kTileK) {
    for (int e = threadIdx.x; e < kTile * kTileK; e += kThreads) {
      const int r = e / kTileK, k = e % kTileK;
      const long long g = row0 + r;
      As[k][r] = (g < G && k0 + k < n) ? ao[g * n + k0 + k] : 0.0;
      const int kk = e / kTile, c = e % kTile;
      Bs[kk][c] = (k0 + kk < n && col0 + c < n) ? D[(long long)(k0 + kk) * n + col0 + c] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kTileK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[k][ty * 4 + q];
        b[q] = Bs[k][tx * 4 + q];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const long long ntile = gridDim.y;
  for (int comp = 0; comp < 4; ++comp) {
    const double* aoc = ao + comp * plane;
    double rp[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long g = row0 + ty * 4 + i;
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = col0 + tx * 4 + j;
        if (g < G && c < n) s = fma(acc[i][j], aoc[g * n + c], s);
      }
      rp[i] = s;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) rp[i] += __shfl_xor_sync(kFull, rp[i], o);
    }
    if (tx == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const long long g = row0 + ty * 4 + i;
        if (g < G) part[(comp * ntile + blockIdx.y) * G + g] = rp[i];
      }
    }
  }
}

// rho = sum of the value partials; grad rho = 2 sum of the derivative partials
__global__ void rho_gga_sum_kernel(long long G, int ntile, const double* __restrict__ part,
                                   double* __restrict__ rho4) {
  const long long total = 4 * G;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long comp = e / G, g = e - comp * G;
    double s = 0.0;
    for (int t = 0; t < ntile; ++t) s += part[(comp * ntile + t) * G + g];
    rho4[e] = comp == 0 ? s : 2.0 * s;
  }
}

// ---------------------------------------------------------------------------
// PBE exchange, spin-unpolarised: e = A rho^(4/3) F(u), u = s^2 = c sigma rho^(-8/3),
// F(u) = 1 + kappa - kappa^2 / (kappa + mu u).  exc = e / rho, and the
// (weighted) GGA potential weights of _rks_gga_wv0:
//   wv0 = 0.5 w de/drho, wv_q = 2 w de/dsigma drho/dq.
// Per-block partial sums of w rho and w e (deterministic).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) pbe_x_kernel(long long G,
                                                         const double* __restrict__ rho4,
                                                         const double* __restrict__ w,
                                                         double* __restrict__ exc,
                                                         double* __restrict__ wv,
                                                         double* __restrict__ part) {
  const double pi = 3.141592653589793;
  const double A = -0.75 * cbrt(3.0 / pi);
  const double kappa = 0.804, mu = 0.2195149727645171;
  const double cs = 1.0 / (4.0 * cbrt(9.0 * pi * pi * pi * pi));  // 1 / (4 (3 pi^2)^(2/3))
  double sn = 0.0, se = 0.0;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (long long)gridDim.x * blockDim.x) {
    const double r = rho4[g];
    const double gx = rho4[G + g], gy = rho4[2 * G + g], gz = rho4[3 * G + g];
    double e = 0.0, vr = 0.0, vs = 0.0, eps = 0.0;
    if (r > 1e-14) {
      const double r13 = cbrt(r);
      const double r43 = r * r13;
      const double sigma = gx * gx + gy * gy + gz * gz;
      const double u = cs * sigma / (r43 * r43);
      const double den = kappa + mu * u;
      const double F = 1.0 + kappa - kappa * kappa / den;
      const double dF = kappa * kappa * mu / (den * den);
      e = A * r43 * F;
      eps = A * r13 * F;
      vr = A * r13 * (4.0 / 3.0 * F - 8.0 / 3.0 * u * dF);
      vs = A * cs * dF / r43;
    }
    const double wg = w[g];
    if (exc) exc[g] = eps;
    wv[g] = 0.5 * wg * vr;
    wv[G + g] = 2.0 * wg * vs * gx;
    wv[2 * G + g] = 2.0 * wg * vs * gy;
    wv[3 * G + g] = 2.0 * wg * vs * gz;
    sn = fma(wg, r, sn);
    se = fma(wg, e, se);
  }
  __shared__ double red[2][kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    sn += __shfl_xor_sync(kFull, sn, o);
    se += __shfl_xor_sync(kFull, se, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = sn;
    red[1][threadIdx.x >> 5] = se;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kThreads / 32; ++k) {
      a += red[0][k];
      b += red[1][k];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

__global__ void pair_sum_kernel(int nblocks, const double* __restrict__ part, double* sums) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nblocks; ++k) {
      a += part[2 * k];
      b += part[2 * k + 1];
    }
    sums[0] = a;
    sums[1] = b;
  }
}

// ---------------------------------------------------------------------------
// M = ao0^T aow, aow_gc = sum_n wv_n,g ao_n,gc: all 64 x 64 tiles (M is not
// symmetric), split over grid chunks; vmat = M + M^T summed over the chunks
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) vxc_gga_kernel(long long G, int n,
                                                           const double* __restrict__ ao,
                                                           const double* __restrict__ wv,
                                                           double* __restrict__ part,
                                                           long long chunk) {
  __shared__ double As[kTileK][kTile + 1];
  __shared__ double Bs[kTileK][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = blockIdx.x * kTile, c0 = blockIdx.y * kTile;
  const long long g0 = (long long)blockIdx.z * chunk;
  const long long g1 = min(G, g0 + chunk);
  const long long plane = G * n;
  double acc[4][4] = {};
  for (long long gk = g0; gk < g1; gk += kTileK) {
    for (int e = threadIdx.x; e < kTile * kTileK; e += kThreads) {
      const int k = e / kTile, c = e % kTile;
      const long long g = gk + k;
      const bool ok = g < g1;
      As[k][c] = (ok && r0 + c < n) ? ao[g * n + r0 + c] : 0.0;
      double b = 0.0;
      if (ok && c0 + c < n) {
        const long long idx = g * n + c0 + c;
#pragma unroll
        for (int q = 0; q < 4; ++q) b = fma(wv[q * G + g], ao[q * plane + idx], b);
      }
      Bs[k][c] = b;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kTileK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[k][ty * 4 + q];
        b[q] = Bs[k][tx * 4 + q];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* P = part + (long long)blockIdx.z * n * n;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = r0 + ty * 4 + i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = c0 + tx * 4 + j;
      if (r < n && c < n) P[(long long)r * n + c] = acc[i][j];
    }
  }
}

__global__ void vxc_gga_sum_kernel(int n, int nchunks, const double* __restrict__ part,
                                   double* __restrict__ vmat) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c)
      s += part[(long long)c * nn + (long long)i * n + j] + part[(long long)c * nn + (long long)j * n + i];
    vmat[e] = s;
  }
}

long long gga_chunk_len(long long G, int nao) {
  const long long tiles = (nao + kTile - 1) / kTile;
  long long chunks = (kCtas + tiles * tiles - 1) / (tiles * tiles);
  long long len = (G + chunks - 1) / chunks;
  len = (len + kTileK - 1) / kTileK * kTileK;
  return len < kTileK ? kTileK : len;
}

constexpr int kPbeBlocks = 608;

}  // namespace

extern "C" {

int qex_td_eval_ao_deriv1(int64_t num_points, const double* coords, int32_t num_shells,
                          const double* centers, const int32_t* l, const int32_t* prim_offset,
                          const int32_t* ao_offset, const double* exponents,
                          const double* coefficients, int32_t nao, double* ao4, void* stream) {
  if (num_points < 0 || num_shells < 0 || nao < 1) return QEX_BAD_ARG;
  if (num_points == 0 || num_shells == 0) return QEX_OK;
  if (!coords || !centers || !l || !prim_offset || !ao_offset || !exponents || !coefficients ||
      !ao4)
    return QEX_BAD_ARG;
  const long long work = num_points * num_shells;
  eval_ao_d1_kernel<<<grid_for(work, kThreads), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      num_points, coords, num_shells, centers, l, prim_offset, ao_offset, exponents, coefficients,
      nao, ao4);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_rho_gga_workspace_size(int64_t num_points, int32_t nao) {
  if (num_points < 0 || nao < 1) return 0;
  return sizeof(double) * 4 * (size_t)num_points * (size_t)((nao + kTile - 1) / kTile);
}

int qex_td_rho_gga(int64_t num_points, int32_t nao, const double* ao4, const double* dm,
                   double* rho4, void* workspace, size_t workspace_bytes, void* stream) {
  if (num_points < 0 || nao < 1) return QEX_BAD_ARG;
  if (num_points == 0) return QEX_OK;
  if (!ao4 || !dm || !rho4 || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_rho_gga_workspace_size(num_points, nao)) return QEX_BAD_ARG;
  const long long rows = (num_points + kTile - 1) / kTile;
  if (rows > 2147483647LL) return QEX_BAD_ARG;
  const int ctiles = (nao + kTile - 1) / kTile;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  rho_gga_kernel<<<dim3((unsigned)rows, ctiles), kThreads, 0, s>>>(num_points, nao, ao4, dm, part);
  rho_gga_sum_kernel<<<grid_for(4 * num_points, kThreads), kThreads, 0, s>>>(num_points, ctiles,
                                                                            part, rho4);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_gga_pbe_x_workspace_size(int64_t num_points) {
  (void)num_points;
  return sizeof(double) * 2 * kPbeBlocks;
}

int qex_td_gga_pbe_x(int64_t num_points, const double* rho4, const double* weights, double* exc,
                     double* wv, double* sums, void* workspace, size_t workspace_bytes,
                     void* stream) {
  if (num_points < 0 || !rho4 || !weights || !wv || !sums || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_gga_pbe_x_workspace_size(num_points)) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  long long blocks = (num_points + kThreads - 1) / kThreads;
  if (blocks > kPbeBlocks) blocks = kPbeBlocks;
  if (blocks < 1) blocks = 1;
  pbe_x_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(num_points, rho4, weights, exc, wv, part);
  pair_sum_kernel<<<1, 32, 0, s>>>((int)blocks, part, sums);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_vxc_gga_workspace_size(int64_t num_points, int32_t nao) {
  if (num_points < 0 || nao < 1) return 0;
  const long long len = gga_chunk_len(num_points, nao);
  const long long chunks = (num_points + len - 1) / len;
  return sizeof(double) * (size_t)(chunks < 1 ? 1 : chunks) * (size_t)nao * (size_t)nao;
}

int qex_td_vxc_gga(int64_t num_points, int32_t nao, const double* ao4, const double* wv,
                   double* vmat, void* workspace, size_t workspace_bytes, void* stream) {
  if (num_points < 0 || nao < 1) return QEX_BAD_ARG;
  if (!ao4 || !wv || !vmat || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_vxc_gga_workspace_size(num_points, nao)) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long len = gga_chunk_len(num_points, nao);
  long long chunks = (num_points + len - 1) / len;
  if (chunks < 1) chunks = 1;
  if (chunks > 65535) return QEX_BAD_ARG;
  double* part = static_cast<double*>(workspace);
  const int tiles = (nao + kTile - 1) / kTile;
  if (num_points == 0) cudaMemsetAsync(part, 0, sizeof(double) * (size_t)nao * nao, s);
  vxc_gga_kernel<<<dim3(tiles, tiles, (unsigned)chunks), kThreads, 0, s>>>(num_points, nao, ao4,
                                                                          wv, part, len);
  vxc_gga_sum_kernel<<<grid_for((long long)nao * nao, kThreads), kThreads, 0, s>>>(
      nao, (int)chunks, part, vmat);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
