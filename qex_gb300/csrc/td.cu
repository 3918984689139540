// GB300 (sm_103a) kernels of the 3D Kohn-Sham numint SCF (FP64).
//
// Reference path (qedft, pasqal-io/qex): qedft/train/td/numint_legacy.py:122-481
// (nr_rks, eval_rho, _scale_ao, _dot_ao_ao), generalized_eigensolver.py:264-330,
// jax_diis.py:26-134, hf.py:303-308 and the fixed-cycle masked SCF of
// scf_functions_masked.py:907-967.  All contractions are deterministic: every
// reduction writes per-block partials that a second pass sums in a fixed order.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "cart.cuh"
#include "ks1d_common.cuh"
#include "qex_ks1d.h"
#include "qex_td.h"

// Mixed-precision generalized eigensolver (eigh_mp.cu).
bool qex_mp_gen_eigh(int batch, int n, const double* A, const double* S, double* w, double* V,
                     int32_t* status, double* area, int* ok_out, cudaStream_t s);
long long qex_mp_area_doubles(int n);
bool qex_mp_set_path(int n, int path);

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTile = 64;      // GEMM tile (rows x cols)
constexpr int kTileK = 16;     // GEMM k-step
constexpr int kThreads = 256;  // 16 x 16 threads, 4 x 4 outputs each
constexpr int kVxcCtas = 304;  // target CTAs of one Vxc product (2 per SM)

// Grid points per Vxc chunk: enough chunks that the upper tiles times the
// chunks fill the GPU (FP64 issues slowly on one SM), at least one k-step.
long long vxc_chunk_len(long long G, int nao) {
  const long long tiles = (nao + kTile - 1) / kTile;
  const long long upper = tiles * (tiles + 1) / 2;
  long long chunks = (kVxcCtas + upper - 1) / upper;
  long long len = (G + chunks - 1) / chunks;
  len = (len + kTileK - 1) / kTileK * kTileK;
  return len < kTileK ? kTileK : len;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Deterministic block reduction (blockDim.x == kThreads).
__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < kThreads / 32) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

int grid_for(long long work, int threads) {
  long long g = (work + threads - 1) / threads;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// AO values
// ---------------------------------------------------------------------------
__global__ void eval_ao_kernel(long long G, const double* __restrict__ coords, int ns,
                               const double* __restrict__ centers, const int* __restrict__ l,
                               const int* __restrict__ poff, const int* __restrict__ aooff,
                               const double* __restrict__ ex, const double* __restrict__ co,
                               int nao, double* __restrict__ ao) {
  const long long total = G * ns;
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const long long g = it / ns;
    const int s = (int)(it - g * ns);
    const double dx = coords[3 * g] - centers[3 * s];
    const double dy = coords[3 * g + 1] - centers[3 * s + 1];
    const double dz = coords[3 * g + 2] - centers[3 * s + 2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    double rad = 0.0;
    for (int p = poff[s]; p < poff[s + 1]; ++p) rad += co[p] * exp(-ex[p] * r2);
    double* row = ao + g * nao + aooff[s];
    const int ls = l[s];
    if (ls < 0 || ls > kMaxShellL) continue;
    for (int k = 0; k < ncart(ls); ++k) {
      int c[3];
      cart_exponents(ls, k, c);
      row[k] = cart_pow(dx, c[0]) * cart_pow(dy, c[1]) * cart_pow(dz, c[2]) * rad;
    }
  }
}

// ---------------------------------------------------------------------------
// rho_g = sum_i (ao D)_gi ao_gi : 64 x 64 output tiles of T = ao D, the row
// dot with ao fused into the epilogue; partials per column tile.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) rho_kernel(long long G, int n,
                                                       const double* __restrict__ ao,
                                                       const double* __restrict__ D,
                                                       double* __restrict__ part) {
  __shared__ double As[kTileK][kTile + 1];
  __shared__ double Bs[kTileK][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long long row0 = (long long)blockIdx.x * kTile;
  const int col0 = blockIdx.y * kTile;
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
  // epilogue: row partial sum_j T_gj ao_gj over this thread's 4 columns,
  // then across the 16 threads of the row group (one half-warp)
  double rp[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const long long g = row0 + ty * 4 + i;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = col0 + tx * 4 + j;
      if (g < G && c < n) s = fma(acc[i][j], ao[g * n + c], s);
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
      if (g < G) part[(long long)blockIdx.y * G + g] = rp[i];
    }
  }
}

__global__ void sum_parts_kernel(long long G, int nparts, const double* __restrict__ part,
                                 double* __restrict__ out) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += part[(long long)p * G + g];
    out[g] = s;
  }
}

// ---------------------------------------------------------------------------
// LDA on the grid: Slater exchange, optionally with the VWN correlation of the
// reference's default "LDA,VWN" (qedft/train/td/rks.py:172; libxc's VWN is the
// paramagnetic fit 5 of Vosko, Wilk and Nusair, Can. J. Phys. 58, 1200 (1980)).
// ---------------------------------------------------------------------------
// eps_c and v_c = d(rho eps_c)/d rho at density r, in Hartree.
__device__ inline void vwn5_c(double r, double& eps, double& v) {
  if (!(r > 1e-30)) {
    eps = 0.0;
    v = 0.0;
    return;
  }
  const double A = 0.0310907, b = 3.72744, c = 12.9352, x0 = -0.10498;
  const double pi = 3.141592653589793;
  const double rs = cbrt(3.0 / (4.0 * pi * r));
  const double x = sqrt(rs);
  const double X = x * x + b * x + c;
  const double X0 = x0 * x0 + b * x0 + c;
  const double Q = sqrt(4.0 * c - b * b);
  const double t = 2.0 * x + b;
  const double at = atan(Q / t);
  const double f = b * x0 / X0;
  eps = A * (log(x * x / X) + 2.0 * b / Q * at -
             f * (log((x - x0) * (x - x0) / X) + 2.0 * (b + 2.0 * x0) / Q * at));
  const double den = t * t + Q * Q;
  const double de_dx = A * (2.0 / x - t / X - 4.0 * b / den -
                            f * (2.0 / (x - x0) - t / X - 4.0 * (b + 2.0 * x0) / den));
  v = eps - x / 6.0 * de_dx;
}

template <bool kVwn>
__global__ void __launch_bounds__(kThreads) lda_kernel(long long G, const double* __restrict__ rho,
                                                       const double* __restrict__ w,
                                                       double* __restrict__ exc,
                                                       double* __restrict__ vrho,
                                                       double* __restrict__ part) {
  __shared__ double red[kThreads / 32];
  const double cx = 0.7385587663820224;  // (3/4) (3/pi)^(1/3)
  double s0 = 0.0, s1 = 0.0;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G;
       g += (long long)gridDim.x * blockDim.x) {
    const double r = rho[g];
    double e = -cx * cbrt(fmax(r, 0.0));
    double v = (4.0 / 3.0) * e;
    if (kVwn) {
      double ec, vc;
      vwn5_c(r, ec, vc);
      e += ec;
      v += vc;
    }
    if (exc) exc[g] = e;
    if (vrho) vrho[g] = v;
    const double den = r * w[g];
    s0 += den;
    s1 = fma(den, e, s1);
  }
  s0 = block_sum(s0, red);
  s1 = block_sum(s1, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s0;
    part[2 * blockIdx.x + 1] = s1;
  }
}

__global__ void lda_sum_kernel(int nblocks, const double* __restrict__ part, double* sums) {
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nblocks; ++i) {
      a += part[2 * i];
      b += part[2 * i + 1];
    }
    sums[0] = a;
    sums[1] = b;
  }
}

// ---------------------------------------------------------------------------
// vmat = ao^T diag(s) ao, s = 0.5 w v: upper tiles, split over grid chunks
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) vxc_kernel(long long G, int n,
                                                       const double* __restrict__ ao,
                                                       const double* __restrict__ w,
                                                       const double* __restrict__ v,
                                                       double* __restrict__ part,
                                                       long long chunk) {
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (ti > tj) return;
  __shared__ double As[kTileK][kTile + 1];
  __shared__ double Bs[kTileK][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = ti * kTile, c0 = tj * kTile;
  const long long g0 = (long long)blockIdx.z * chunk;
  const long long g1 = min(G, g0 + chunk);
  double acc[4][4] = {};
  for (long long gk = g0; gk < g1; gk += kTileK) {
    for (int e = threadIdx.x; e < kTile * kTileK; e += kThreads) {
      const int k = e / kTile, c = e % kTile;
      const long long g = gk + k;
      const bool ok = g < g1;
      const double sg = ok ? 0.5 * w[g] * v[g] : 0.0;
      As[k][c] = (ok && r0 + c < n) ? ao[g * n + r0 + c] * sg : 0.0;
      Bs[k][c] = (ok && c0 + c < n) ? ao[g * n + c0 + c] : 0.0;
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

__global__ void vxc_sum_kernel(int n, int nchunks, const double* __restrict__ part,
                               double* __restrict__ vmat) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    int i = (int)(e / n), j = (int)(e % n);
    // only tiles with tile(i) <= tile(j) were computed; the matrix is symmetric
    int a = i, b = j;
    if (i / kTile > j / kTile) {
      a = j;
      b = i;
    }
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += part[(long long)c * nn + (long long)a * n + b];
    vmat[e] = 2.0 * s;  // vmat + vmat^T of the symmetric half-weight matrix
  }
}

// ---------------------------------------------------------------------------
// Small dense helpers
// ---------------------------------------------------------------------------
// C = A B for n x n row-major matrices (32 x 32 tiles)
__global__ void gemm_nn_kernel(int n, const double* __restrict__ A, const double* __restrict__ B,
                               double* __restrict__ C) {
  __shared__ double As[32][33];
  __shared__ double Bs[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  const int row0 = blockIdx.y * 32, col0 = blockIdx.x * 32;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k0 = 0; k0 < n; k0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      As[r][tx] = (row0 + r < n && k0 + tx < n) ? A[(long long)(row0 + r) * n + k0 + tx] : 0.0;
      Bs[r][tx] = (k0 + r < n && col0 + tx < n) ? B[(long long)(k0 + r) * n + col0 + tx] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const double b = Bs[k][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(As[ty + 8 * q][k], b, acc[q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = row0 + ty + 8 * q, c = col0 + tx;
    if (r < n && c < n) C[(long long)r * n + c] = acc[q];
  }
}

__global__ void antisym_kernel(int n, const double* __restrict__ Y, double* __restrict__ E) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    E[e] = Y[e] - Y[(long long)j * n + i];
  }
}

__global__ void make_rdm1_kernel(int batch, int n, const double* __restrict__ C,
                                 const double* __restrict__ occ, double* __restrict__ D) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn * batch;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / nn;
    const long long r = e - b * nn;
    const int i = (int)(r / n), j = (int)(r % n);
    const double* Cb = C + b * nn;
    const double* ob = occ + b * n;
    double s = 0.0;
    for (int k = 0; k < n; ++k) {
      const double o = ob[k];
      if (o > 0.0) s = fma(o * Cb[(long long)i * n + k], Cb[(long long)j * n + k], s);
    }
    D[e] = s;
  }
}

// ---------------------------------------------------------------------------
// DIIS extrapolation (one CTA)
// ---------------------------------------------------------------------------
constexpr int kMaxDiis = 16;
__global__ void __launch_bounds__(kThreads) diis_kernel(int n, int nvec, int min_vecs,
                                                        const double* __restrict__ errs,
                                                        const double* __restrict__ focks,
                                                        double* __restrict__ out,
                                                        double* __restrict__ coeffs) {
  __shared__ double red[kThreads / 32];
  __shared__ double Bm[kMaxDiis + 1][kMaxDiis + 2];
  __shared__ double c[kMaxDiis + 1];
  const long long nn = (long long)n * n;
  if (nvec < min_vecs) {
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) out[e] = focks[(long long)(nvec - 1) * nn + e];
    return;
  }
  for (int i = 0; i < nvec; ++i) {
    for (int j = i; j < nvec; ++j) {
      double s = 0.0;
      for (long long e = threadIdx.x; e < nn; e += blockDim.x)
        s = fma(errs[(long long)i * nn + e], errs[(long long)j * nn + e], s);
      s = block_sum(s, red);
      if (threadIdx.x == 0) {
        Bm[i + 1][j + 1] = s;
        Bm[j + 1][i + 1] = s;
      }
    }
  }
  if (threadIdx.x == 0) {
    const int m = nvec + 1;
    Bm[0][0] = 0.0;
    for (int i = 1; i < m; ++i) {
      Bm[0][i] = -1.0;
      Bm[i][0] = -1.0;
    }
    for (int i = 0; i < m; ++i) {
      Bm[i][i] += 1e-14;
      Bm[i][m] = (i == 0) ? -1.0 : 0.0;  // right-hand side
    }
    // Gaussian elimination with partial pivoting
    for (int k = 0; k < m; ++k) {
      int piv = k;
      for (int i = k + 1; i < m; ++i)
        if (fabs(Bm[i][k]) > fabs(Bm[piv][k])) piv = i;
      if (piv != k)
        for (int j = 0; j <= m; ++j) {
          double t = Bm[k][j];
          Bm[k][j] = Bm[piv][j];
          Bm[piv][j] = t;
        }
      const double d = Bm[k][k];
      for (int i = k + 1; i < m; ++i) {
        const double f = (d != 0.0) ? Bm[i][k] / d : 0.0;
        for (int j = k; j <= m; ++j) Bm[i][j] -= f * Bm[k][j];
      }
    }
    for (int i = m - 1; i >= 0; --i) {
      double s = Bm[i][m];
      for (int j = i + 1; j < m; ++j) s -= Bm[i][j] * c[j];
      c[i] = (Bm[i][i] != 0.0) ? s / Bm[i][i] : 0.0;
    }
    if (coeffs)
      for (int i = 0; i < nvec; ++i) coeffs[i] = c[i + 1];
  }
  __syncthreads();
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < nvec; ++i) s = fma(c[i + 1], focks[(long long)i * nn + e], s);
    out[e] = s;
  }
}

// ---------------------------------------------------------------------------
// Coulomb from factored ERIs
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) coul_contract_kernel(int n, const double* __restrict__ Bf,
                                                                 const double* __restrict__ D,
                                                                 double* __restrict__ cvec) {
  __shared__ double red[kThreads / 32];
  const long long nn = (long long)n * n;
  const double* Bp = Bf + (long long)blockIdx.x * nn;
  double s = 0.0;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) s = fma(Bp[e], D[e], s);
  s = block_sum(s, red);
  if (threadIdx.x == 0) cvec[blockIdx.x] = s;
}

__global__ void coul_expand_kernel(int n, int naux, const double* __restrict__ Bf,
                                   const double* __restrict__ cvec, double* __restrict__ J) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < naux; ++p) s = fma(cvec[p], Bf[(long long)p * nn + e], s);
    J[e] = s;
  }
}

// ---------------------------------------------------------------------------
// Generalized eigensolver: one CTA per matrix.  Cholesky of S, C = L^-1 A L^-T
// by triangular solves, parallel cyclic Jacobi on C (round-robin pairing),
// V = L^-T U, ascending sort.
// ---------------------------------------------------------------------------
constexpr int kEighThreads = 512;
constexpr int kMaxSweeps = 30;

struct EighWork {
  double* L;
  double* C;
  double* U;
  double* t;  // n
  int* perm;  // n (+1)
};

__device__ bool cholesky(int n, double* L, double* flag_shared) {
  // in place: lower triangle of L holds S on entry, its Cholesky factor on exit
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      double d = L[(long long)k * n + k];
      flag_shared[0] = d;
      L[(long long)k * n + k] = d > 0.0 ? sqrt(d) : 0.0;
    }
    __syncthreads();
    if (!(flag_shared[0] > 0.0)) return false;
    const double lkk = L[(long long)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) L[(long long)i * n + k] /= lkk;
    __syncthreads();
    const int m = n - k - 1;
    for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
      const int i = k + 1 + (int)(e / m), j = k + 1 + (int)(e % m);
      if (j <= i) L[(long long)i * n + j] -= L[(long long)i * n + k] * L[(long long)j * n + k];
    }
    __syncthreads();
  }
  for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j > i) L[e] = 0.0;
  }
  __syncthreads();
  return true;
}

// Parallel cyclic Jacobi on symmetric C (global, n x n); accumulates U.
// Returns the number of sweeps used (kMaxSweeps + 1 if not converged).
__device__ int jacobi(int n, double* C, double* U, int* pos, double* cs, int* pq, double* red) {
  const int m = (n + 1) & ~1;  // even number of slots (a dummy when n is odd)
  for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    U[e] = (i == j) ? 1.0 : 0.0;
  }
  for (int i = threadIdx.x; i < m; i += blockDim.x) pos[i] = i;
  __syncthreads();
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
      const int i = (int)(e / n), j = (int)(e % n);
      const double v = C[e];
      if (i == j) {
        dia = fma(v, v, dia);
      } else {
        off = fma(v, v, off);
      }
    }
    off = block_sum(off, red);
    dia = block_sum(dia, red);
    // converged when the off-diagonal norm is 1e-14 of the diagonal (the FP64 floor is ~1e-16)
    if (off <= 1e-28 * dia || off == 0.0) return sweep;
    for (int step = 0; step < m - 1; ++step) {
      // pairs of this round-robin step
      for (int k = threadIdx.x; k < m / 2; k += blockDim.x) {
        int p = pos[k], q = pos[m - 1 - k];
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = C[(long long)p * n + q];
          if (apq != 0.0) {
            // rotation angle in FP32 (it need not annihilate a_pq exactly: the
            // sweeps converge all the same), made orthogonal in FP64
            const double app = C[(long long)p * n + p], aqq = C[(long long)q * n + q];
            const float th = __fdividef((float)(aqq - app), 2.0f * (float)apq);
            const float t = (fabsf(th) < 1e18f)
                                ? copysignf(1.0f, th) / (fabsf(th) + sqrtf(fmaf(th, th, 1.0f)))
                                : 0.0f;
            if (t != 0.0f) {
              const float cf = rsqrtf(fmaf(t, t, 1.0f));
              c = (double)cf;
              s = (double)(t * cf);
              const double nrm = qex::rsqrt_nr(fma(c, c, s * s));
              c *= nrm;
              s *= nrm;
            }
          }
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
        pq[2 * k] = p;
        pq[2 * k + 1] = q;
      }
      __syncthreads();
      // rows p, q <- J^T rows
      for (long long e = threadIdx.x; e < (long long)(m / 2) * n; e += blockDim.x) {
        const int k = (int)(e / n), j = (int)(e % n);
        const double s = cs[2 * k + 1];
        if (s == 0.0) continue;
        const double c = cs[2 * k];
        const int p = pq[2 * k], q = pq[2 * k + 1];
        const double xp = C[(long long)p * n + j], xq = C[(long long)q * n + j];
        C[(long long)p * n + j] = c * xp - s * xq;
        C[(long long)q * n + j] = s * xp + c * xq;
      }
      __syncthreads();
      // columns p, q of C and U <- J columns
      for (long long e = threadIdx.x; e < (long long)(m / 2) * n; e += blockDim.x) {
        const int k = (int)(e / n), i = (int)(e % n);
        const double s = cs[2 * k + 1];
        if (s == 0.0) continue;
        const double c = cs[2 * k];
        const int p = pq[2 * k], q = pq[2 * k + 1];
        double xp = C[(long long)i * n + p], xq = C[(long long)i * n + q];
        C[(long long)i * n + p] = c * xp - s * xq;
        C[(long long)i * n + q] = s * xp + c * xq;
        xp = U[(long long)i * n + p];
        xq = U[(long long)i * n + q];
        U[(long long)i * n + p] = c * xp - s * xq;
        U[(long long)i * n + q] = s * xp + c * xq;
      }
      __syncthreads();
      // round-robin rotation of positions 1..m-1
      if (threadIdx.x == 0) {
        const int last = pos[m - 1];
        for (int i = m - 1; i > 1; --i) pos[i] = pos[i - 1];
        pos[1] = last;
      }
      __syncthreads();
    }
  }
  return kMaxSweeps + 1;
}

__global__ void __launch_bounds__(kEighThreads) gen_eigh_kernel(int n, const double* __restrict__ A,
                                                                const double* __restrict__ S,
                                                                double* __restrict__ w,
                                                                double* __restrict__ V,
                                                                int* __restrict__ status,
                                                                double* __restrict__ ws,
                                                                const int* __restrict__ done) {
  if (done && done[blockIdx.x]) return;  // solved by the mixed-precision path
  __shared__ double red[kEighThreads / 32];
  __shared__ double flag[2];
  extern __shared__ double dyn[];  // cs (2 * m/2), pos (m), pq (m) ints
  const int m = (n + 1) & ~1;
  double* cs = dyn;
  int* pos = reinterpret_cast<int*>(cs + m);
  int* pq = pos + m;
  int* perm = pq + m;
  const int b = blockIdx.x;
  const long long nn = (long long)n * n;
  const double* Ab = A + b * nn;
  const double* Sb = S + b * nn;
  double* L = ws + (long long)b * 3 * nn;
  double* C = L + nn;
  double* U = C + nn;
  int st = 0;
  // symmetrise inputs: C <- (A + A^T)/2, L <- (S + S^T)/2
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    C[e] = 0.5 * (Ab[e] + Ab[(long long)j * n + i]);
    L[e] = 0.5 * (Sb[e] + Sb[(long long)j * n + i]);
  }
  __syncthreads();
  if (!cholesky(n, L, flag)) {
    // S is not numerically SPD: shift by (1e-12 - lambda_min(S)) as the
    // reference does, with lambda_min from a Jacobi diagonalisation of S
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
      const int i = (int)(e / n), j = (int)(e % n);
      V[b * nn + e] = 0.5 * (Sb[e] + Sb[(long long)j * n + i]);
    }
    __syncthreads();
    jacobi(n, V + b * nn, U, pos, cs, pq, red);
    if (threadIdx.x == 0) {
      double lmin = 1e300;
      for (int i = 0; i < n; ++i) lmin = fmin(lmin, V[b * nn + (long long)i * n + i]);
      flag[1] = (lmin < 1e-12) ? (1e-12 - lmin) : 0.0;
    }
    __syncthreads();
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
      const int i = (int)(e / n), j = (int)(e % n);
      L[e] = 0.5 * (Sb[e] + Sb[(long long)j * n + i]) + (i == j ? flag[1] : 0.0);
    }
    __syncthreads();
    st = QEX_NUMERICAL;
    if (!cholesky(n, L, flag)) {
      if (threadIdx.x == 0 && status) status[b] = QEX_NUMERICAL;
      return;
    }
  }
  // C <- L^-1 C (forward substitution, one column per thread)
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      double s = C[(long long)i * n + j];
      for (int k = 0; k < i; ++k) s -= L[(long long)i * n + k] * C[(long long)k * n + j];
      C[(long long)i * n + j] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  // C <- C L^-T: row r of the result solves L y = row r of C
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      double s = C[(long long)r * n + i];
      for (int k = 0; k < i; ++k) s -= L[(long long)i * n + k] * C[(long long)r * n + k];
      C[(long long)r * n + i] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j > i) {
      const double v = 0.5 * (C[e] + C[(long long)j * n + i]);
      C[e] = v;
      C[(long long)j * n + i] = v;
    }
  }
  __syncthreads();
  const int sweeps = jacobi(n, C, U, pos, cs, pq, red);
  if (sweeps > kMaxSweeps) st = QEX_NOT_CONVERGED;
  // V = L^-T U (back substitution, one column per thread), unsorted in V
  double* Vb = V + b * nn;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = n - 1; i >= 0; --i) {
      double s = U[(long long)i * n + j];
      for (int k = i + 1; k < n; ++k) s -= L[(long long)k * n + i] * Vb[(long long)k * n + j];
      Vb[(long long)i * n + j] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  // ascending order of the eigenvalues (stable selection by rank)
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double di = C[(long long)i * n + i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double dj = C[(long long)j * n + j];
      rank += (dj < di) || (dj == di && j < i);
    }
    perm[rank] = i;
  }
  __syncthreads();
  // permute columns through U (free now)
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) U[e] = Vb[e];
  __syncthreads();
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), r = (int)(e % n);
    Vb[e] = U[(long long)i * n + perm[r]];
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) w[(long long)b * n + r] = C[(long long)perm[r] * n + perm[r]];
  if (threadIdx.x == 0 && status) status[b] = st;
}

}  // namespace

extern "C" {

int qex_td_eval_ao(int64_t num_points, const double* coords, int32_t num_shells,
                   const double* centers, const int32_t* l, const int32_t* prim_offset,
                   const int32_t* ao_offset, const double* exponents, const double* coefficients,
                   int32_t nao, double* ao, void* stream) {
  if (num_points < 0 || num_shells < 0 || nao < 1) return QEX_BAD_ARG;
  if (num_points == 0 || num_shells == 0) return QEX_OK;
  if (!coords || !centers || !l || !prim_offset || !ao_offset || !exponents || !coefficients || !ao)
    return QEX_BAD_ARG;
  const long long work = (long long)num_points * num_shells;
  eval_ao_kernel<<<grid_for(work, kThreads), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      num_points, coords, num_shells, centers, l, prim_offset, ao_offset, exponents, coefficients,
      nao, ao);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_rho_workspace_size(int64_t num_points, int32_t nao) {
  if (num_points < 0 || nao < 1) return 0;
  return sizeof(double) * (size_t)num_points * (size_t)((nao + kTile - 1) / kTile);
}

int qex_td_rho(int64_t num_points, int32_t nao, const double* ao, const double* dm, double* rho,
               void* workspace, size_t workspace_bytes, void* stream) {
  if (num_points < 0 || nao < 1) return QEX_BAD_ARG;
  if (num_points == 0) return QEX_OK;
  if (!ao || !dm || !rho || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_rho_workspace_size(num_points, nao)) return QEX_BAD_ARG;
  const long long rows = (num_points + kTile - 1) / kTile;
  if (rows > 2147483647LL) return QEX_BAD_ARG;
  const int ctiles = (nao + kTile - 1) / kTile;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  rho_kernel<<<dim3((unsigned)rows, ctiles), kThreads, 0, s>>>(num_points, nao, ao, dm, part);
  sum_parts_kernel<<<grid_for(num_points, kThreads), kThreads, 0, s>>>(num_points, ctiles, part, rho);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_lda_workspace_size(int64_t num_points) {
  (void)num_points;
  return sizeof(double) * 2 * 1024;
}

namespace {
int lda_launch(bool vwn, int64_t num_points, const double* rho, const double* weights, double* exc,
               double* vrho, double* sums, void* workspace, size_t workspace_bytes, void* stream) {
  if (num_points < 0) return QEX_BAD_ARG;
  if (!rho || !weights || !sums || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_lda_workspace_size(num_points)) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int blocks = grid_for(num_points, kThreads);
  if (blocks > 1024) blocks = 1024;
  double* part = static_cast<double*>(workspace);
  if (vwn) {
    lda_kernel<true><<<blocks, kThreads, 0, s>>>(num_points, rho, weights, exc, vrho, part);
  } else {
    lda_kernel<false><<<blocks, kThreads, 0, s>>>(num_points, rho, weights, exc, vrho, part);
  }
  lda_sum_kernel<<<1, 32, 0, s>>>(blocks, part, sums);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}
}  // namespace

int qex_td_lda(int64_t num_points, const double* rho, const double* weights, double* exc,
               double* vrho, double* sums, void* workspace, size_t workspace_bytes, void* stream) {
  return lda_launch(false, num_points, rho, weights, exc, vrho, sums, workspace, workspace_bytes,
                    stream);
}

int qex_td_lda_vwn(int64_t num_points, const double* rho, const double* weights, double* exc,
                   double* vrho, double* sums, void* workspace, size_t workspace_bytes,
                   void* stream) {
  return lda_launch(true, num_points, rho, weights, exc, vrho, sums, workspace, workspace_bytes,
                    stream);
}

size_t qex_td_vxc_workspace_size(int64_t num_points, int32_t nao) {
  if (num_points < 0 || nao < 1) return 0;
  const long long len = vxc_chunk_len(num_points, nao);
  const long long chunks = (num_points + len - 1) / len;
  return sizeof(double) * (size_t)(chunks < 1 ? 1 : chunks) * (size_t)nao * (size_t)nao;
}

int qex_td_vxc(int64_t num_points, int32_t nao, const double* ao, const double* weights,
               const double* vrho, double* vmat, void* workspace, size_t workspace_bytes,
               void* stream) {
  if (num_points < 0 || nao < 1) return QEX_BAD_ARG;
  if (!ao || !weights || !vrho || !vmat || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_vxc_workspace_size(num_points, nao)) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long len = vxc_chunk_len(num_points, nao);
  long long chunks = (num_points + len - 1) / len;
  if (chunks < 1) chunks = 1;
  if (chunks > 65535) return QEX_BAD_ARG;
  double* part = static_cast<double*>(workspace);
  const int tiles = (nao + kTile - 1) / kTile;
  if (num_points == 0) cudaMemsetAsync(part, 0, sizeof(double) * (size_t)nao * nao, s);
  vxc_kernel<<<dim3(tiles, tiles, (unsigned)chunks), kThreads, 0, s>>>(num_points, nao, ao, weights,
                                                                       vrho, part, len);
  vxc_sum_kernel<<<grid_for((long long)nao * nao, kThreads), kThreads, 0, s>>>(nao, (int)chunks,
                                                                               part, vmat);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_gen_eigh_workspace_size(int32_t batch, int32_t n) {
  if (batch < 0 || n < 1) return 0;
  // FP64 path (L, C, U), then the mixed-precision area and its ok flags
  return sizeof(double) * (3 * (size_t)n * n + (size_t)qex_mp_area_doubles(n)) * (size_t)batch +
         sizeof(int) * (size_t)batch;
}

int qex_td_gen_eigh_set_path(int32_t n, int32_t path) {
  return qex_mp_set_path(n, path) ? QEX_OK : QEX_BAD_ARG;
}

int qex_td_gen_eigh(int32_t batch, int32_t n, const double* A, const double* S, double* w,
                    double* V, int32_t* status, void* workspace, size_t workspace_bytes,
                    void* stream) {
  if (batch < 0 || n < 1 || n > 4096) return QEX_BAD_ARG;
  if (batch == 0) return QEX_OK;
  if (!A || !S || !w || !V || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_gen_eigh_workspace_size(batch, n)) return QEX_BAD_ARG;
  const int m = (n + 1) & ~1;
  const size_t smem = sizeof(double) * m + sizeof(int) * (3 * m + 2);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* fp64_ws = static_cast<double*>(workspace);
  double* area = fp64_ws + 3 * (size_t)n * n * (size_t)batch;
  int* ok = reinterpret_cast<int*>(area + (size_t)qex_mp_area_doubles(n) * (size_t)batch);
  // FP32 solve + FP64 refinement; the FP64 Jacobi path takes the matrices it
  // leaves (S not numerically SPD, or n beyond its shared memory)
  const bool mp = qex_mp_gen_eigh(batch, n, A, S, w, V, status, area, ok, s);
  gen_eigh_kernel<<<batch, kEighThreads, smem, s>>>(n, A, S, w, V, status, fp64_ws,
                                                    mp ? ok : nullptr);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_make_rdm1(int32_t batch, int32_t n, const double* C, const double* occ, double* D,
                     void* stream) {
  if (batch < 0 || n < 1) return QEX_BAD_ARG;
  if (batch == 0) return QEX_OK;
  if (!C || !occ || !D) return QEX_BAD_ARG;
  const long long work = (long long)batch * n * n;
  make_rdm1_kernel<<<grid_for(work, kThreads), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      batch, n, C, occ, D);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_diis_error(int32_t n, const double* F, const double* D, const double* S, double* err,
                      void* workspace, size_t workspace_bytes, void* stream) {
  if (n < 1 || !F || !D || !S || !err || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < sizeof(double) * (size_t)n * n * 2) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* X = static_cast<double*>(workspace);
  double* Y = X + (size_t)n * n;
  const dim3 grid((n + 31) / 32, (n + 31) / 32);
  gemm_nn_kernel<<<grid, 256, 0, s>>>(n, D, S, X);  // X = D S
  gemm_nn_kernel<<<grid, 256, 0, s>>>(n, F, X, Y);  // Y = F D S
  antisym_kernel<<<grid_for((long long)n * n, kThreads), kThreads, 0, s>>>(n, Y, err);  // FDS - SDF
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_diis_extrapolate(int32_t n, int32_t nvec, int32_t min_vecs, const double* errs,
                            const double* focks, double* fock_out, double* coeffs, void* stream) {
  if (n < 1 || nvec < 1 || nvec > kMaxDiis || !errs || !focks || !fock_out) return QEX_BAD_ARG;
  diis_kernel<<<1, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(n, nvec, min_vecs, errs, focks,
                                                                     fock_out, coeffs);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_coulomb(int32_t n, int32_t naux, const double* factors, const double* dm, double* J,
                   void* workspace, size_t workspace_bytes, void* stream) {
  if (n < 1 || naux < 1 || !factors || !dm || !J || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < sizeof(double) * (size_t)naux) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* cvec = static_cast<double*>(workspace);
  coul_contract_kernel<<<naux, kThreads, 0, s>>>(n, factors, dm, cvec);
  coul_expand_kernel<<<grid_for((long long)n * n, kThreads), kThreads, 0, s>>>(n, naux, factors,
                                                                               cvec, J);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
