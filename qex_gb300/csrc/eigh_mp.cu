// Mixed-precision generalized symmetric eigensolver A x = lambda S x (FP64
// results) for the 3D SCF.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and a one-CTA FP64 Jacobi is
// bound by that pipe on one SM.  So:
//   1. FP32, one CTA per matrix, everything in shared memory: Cholesky S = L L^T,
//      C = L^-1 A L^-T, cyclic Jacobi C = U diag U^T, X = L^-T U.
//   2. FP64 refinement of X (Ogita & Aishima's iterative refinement for the
//      symmetric eigenproblem, in its generalized form): R = I - X^T S X,
//      T = X^T A X, lambda_i = t_ii / (1 - r_ii),
//      e_ij = (t_ij + lambda_j r_ij) / (lambda_j - lambda_i) when the two
//      eigenvalues are further apart than delta = 2 (|T - D|_F + |A|_F |R|_F),
//      else r_ij / 2; X <- X + X E.  Each step squares the error (FP32 ~1e-7
//      times the conditioning of S -> its square -> the FP64 floor); four
//      steps follow the FP32 solve, the last one checked.  The products are
//      batched split-K FP64 GEMMs over many CTAs.
//   3. Ascending order (stable), eigenvectors in columns.
// Overlaps whose FP32 Cholesky fails or whose pivots spread beyond 1e5 take a
// stage 1 with the factor and the transformation in FP64 (the Jacobi stays
// FP32); so does every matrix with n > 128 (up to 240), whose FP32 C alone
// stays in shared memory while the rotations accumulate transposed in global
// memory.  Matrices that are not numerically SPD even in FP64, or that the
// check of the last refinement step rejects, keep the FP64 Jacobi path of
// td.cu, which applies the reference's shift
// (qedft/train/td/generalized_eigensolver.py:264-330).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <atomic>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "qex_ks1d.h"

namespace qex_mp {

constexpr int kThreads = 512;
constexpr int kMaxSweeps32 = 24;
constexpr int kT = 32;      // GEMM tile
constexpr int kKC = 16;     // split-K chunk (one shared-memory stage)
constexpr int kGThreads = 256;
constexpr int kRefineSteps = 4;  // FP32 start -> three squarings -> checked final step

__device__ inline float block_sumf(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.0f;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  __syncthreads();
  return s;
}

__device__ inline double block_max(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = fmax(s, red[i]);
  __syncthreads();
  return s;
}

__device__ inline double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  __syncthreads();
  return s;
}

// Parallel cyclic Jacobi (round-robin pairs) in FP32 on the symmetric C (n x n,
// shared memory); U (set to I by the caller) accumulates the rotations.  With
// kUT, U is stored transposed (row p of U^T is column p of U), so the rotation
// of its columns p, q walks two contiguous rows: the layout for U in global
// memory when n is beyond what shared memory holds.
template <bool kUT>
__device__ void jacobi32(int n, float* C, float* U, float* cs, int* pq, float* red) {
  const long long nn = (long long)n * n;
  const int m = (n + 1) & ~1;
  for (int sweep = 0; sweep < kMaxSweeps32; ++sweep) {
    float off = 0.0f, dia = 0.0f;
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
      const int i = (int)(e / n), j = (int)(e % n);
      const float v = C[e];
      if (i == j) {
        dia = fmaf(v, v, dia);
      } else {
        off = fmaf(v, v, off);
      }
    }
    off = block_sumf(off, red);
    dia = block_sumf(dia, red);
    // FP32 floor: the off-diagonal at ~1e-6 of the diagonal (the FP64
    // refinement takes it from there)
    if (off <= 1e-12f * dia || off == 0.0f) break;
    for (int step = 0; step < m - 1; ++step) {
      for (int k = threadIdx.x; k < m / 2; k += blockDim.x) {
        // round-robin pairing at this step: slot 0 fixed, the others rotated
        // `step` places (closed form of rotating the slot array each step)
        auto slot = [&](int i) { return i == 0 ? 0 : 1 + (i - 1 + (m - 1) - step % (m - 1)) % (m - 1); };
        int p = slot(k), q = slot(m - 1 - k);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        float c = 1.0f, s = 0.0f;
        if (q < n) {
          const float apq = C[(long long)p * n + q];
          if (apq != 0.0f) {
            const float th = (C[(long long)q * n + q] - C[(long long)p * n + p]) / (2.0f * apq);
            const float t = (fabsf(th) < 1e18f)
                                ? copysignf(1.0f, th) / (fabsf(th) + sqrtf(fmaf(th, th, 1.0f)))
                                : 0.0f;
            c = rsqrtf(fmaf(t, t, 1.0f));
            s = t * c;
          }
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
        pq[2 * k] = p;
        pq[2 * k + 1] = q;
      }
      __syncthreads();
      for (long long e = threadIdx.x; e < (long long)(m / 2) * n; e += blockDim.x) {
        const int k = (int)(e / n), j = (int)(e % n);
        const float s = cs[2 * k + 1];
        if (s == 0.0f) continue;
        const float c = cs[2 * k];
        const int p = pq[2 * k], q = pq[2 * k + 1];
        const float xp = C[(long long)p * n + j], xq = C[(long long)q * n + j];
        C[(long long)p * n + j] = c * xp - s * xq;
        C[(long long)q * n + j] = s * xp + c * xq;
      }
      __syncthreads();
      for (long long e = threadIdx.x; e < (long long)(m / 2) * n; e += blockDim.x) {
        const int k = (int)(e / n), i = (int)(e % n);
        const float s = cs[2 * k + 1];
        if (s == 0.0f) continue;
        const float c = cs[2 * k];
        const int p = pq[2 * k], q = pq[2 * k + 1];
        float xp = C[(long long)i * n + p], xq = C[(long long)i * n + q];
        C[(long long)i * n + p] = c * xp - s * xq;
        C[(long long)i * n + q] = s * xp + c * xq;
        const long long up = kUT ? (long long)p * n + i : (long long)i * n + p;
        const long long uq = kUT ? (long long)q * n + i : (long long)i * n + q;
        xp = U[up];
        xq = U[uq];
        U[up] = c * xp - s * xq;
        U[uq] = s * xp + c * xq;
      }
      __syncthreads();
    }
  }
}

// Stage 1: FP32 solve in shared memory.  X (n x n, FP64) receives L^-T U;
// ok[b] = 1 on success, 0 when the FP32 Cholesky of S fails.
__global__ void __launch_bounds__(kThreads) eigh32_kernel(int n, const double* __restrict__ A,
                                                          const double* __restrict__ S,
                                                          double* __restrict__ X,
                                                          int* __restrict__ ok) {
  extern __shared__ float sm[];
  const int b = blockIdx.x;
  const long long nn = (long long)n * n;
  const int m = (n + 1) & ~1;
  float* L = sm;
  float* C = L + nn;
  float* U = C + nn;
  float* cs = U + nn;                                // 2 * (m / 2)
  int* pq = reinterpret_cast<int*>(cs + m);          // m
  float* red = reinterpret_cast<float*>(pq + m);     // 32
  float* piv = red + 32;                             // 3
  const double* Ab = A + b * nn;
  const double* Sb = S + b * nn;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    C[e] = (float)(0.5 * (Ab[e] + Ab[(long long)j * n + i]));
    L[e] = (float)(0.5 * (Sb[e] + Sb[(long long)j * n + i]));
  }
  __syncthreads();
  // Cholesky (right-looking), lower triangle of L; piv[1], piv[2] track the
  // smallest and largest pivot (a lower bound of the conditioning of S)
  if (threadIdx.x == 0) {
    piv[1] = 3e38f;
    piv[2] = 0.0f;
  }
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const float d = L[(long long)k * n + k];
      piv[0] = d;
      piv[1] = fminf(piv[1], d);
      piv[2] = fmaxf(piv[2], d);
      L[(long long)k * n + k] = d > 0.0f ? sqrtf(d) : 0.0f;
    }
    __syncthreads();
    if (!(piv[0] > 0.0f)) {
      if (threadIdx.x == 0) ok[b] = 0;
      return;
    }
    const float inv = 1.0f / L[(long long)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) L[(long long)i * n + k] *= inv;
    __syncthreads();
    const int r = n - k - 1;
    for (long long e = threadIdx.x; e < (long long)r * r; e += blockDim.x) {
      const int i = k + 1 + (int)(e / r), j = k + 1 + (int)(e % r);
      if (j <= i) L[(long long)i * n + j] -= L[(long long)i * n + k] * L[(long long)j * n + k];
    }
    __syncthreads();
  }
  // pivots spread beyond 1e5: the FP32 factor would leave the refinement too
  // far from the solution; the FP64-factor stage takes this matrix
  if (piv[1] < 1e-5f * piv[2]) {
    if (threadIdx.x == 0) ok[b] = 0;
    return;
  }
  // C <- L^-1 C (column j per thread), then C <- C L^-T (row r per thread)
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      float s = C[(long long)i * n + j];
      for (int k = 0; k < i; ++k) s = fmaf(-L[(long long)i * n + k], C[(long long)k * n + j], s);
      C[(long long)i * n + j] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      float s = C[(long long)r * n + i];
      for (int k = 0; k < i; ++k) s = fmaf(-L[(long long)i * n + k], C[(long long)r * n + k], s);
      C[(long long)r * n + i] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j > i) {
      const float v = 0.5f * (C[e] + C[(long long)j * n + i]);
      C[e] = v;
      C[(long long)j * n + i] = v;
    }
    U[e] = (i == j) ? 1.0f : 0.0f;
  }
  __syncthreads();
  jacobi32<false>(n, C, U, cs, pq, red);
  // X = L^-T U: column j solves L^T x = u_j (back substitution)
  double* Xb = X + b * nn;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = n - 1; i >= 0; --i) {
      float s = U[(long long)i * n + j];
      for (int k = i + 1; k < n; ++k) s = fmaf(-L[(long long)k * n + i], U[(long long)k * n + j], s);
      U[(long long)i * n + j] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) Xb[e] = (double)U[e];
  if (threadIdx.x == 0) ok[b] = 1;
}

// Stage 1 for overlaps whose FP32 Cholesky fails (or whose FP32 solve the
// refinement check rejected): S = L L^T and C = L^-1 A L^-T in FP64 (global
// workspace), the Jacobi of C in FP32, X = L^-T U in FP64.  Runs where
// ok[b] == 0 and sets ok[b] = 2 on success (S numerically SPD in FP64).
__global__ void __launch_bounds__(kThreads) eigh32_fp64factor_kernel(
    int n, const double* __restrict__ A, const double* __restrict__ S, double* __restrict__ X,
    double* __restrict__ L64, double* __restrict__ C64, int* __restrict__ ok) {
  const int b = blockIdx.x;
  if (ok[b]) return;
  extern __shared__ float sm[];
  __shared__ double piv;
  const long long nn = (long long)n * n;
  const int m = (n + 1) & ~1;
  float* C = sm;
  float* U = C + nn;
  float* cs = U + nn;
  int* pq = reinterpret_cast<int*>(cs + m);
  float* red = reinterpret_cast<float*>(pq + m);
  double* L = L64 + b * nn;
  double* Cd = C64 + b * nn;
  const double* Ab = A + b * nn;
  const double* Sb = S + b * nn;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    Cd[e] = 0.5 * (Ab[e] + Ab[(long long)j * n + i]);
    L[e] = 0.5 * (Sb[e] + Sb[(long long)j * n + i]);
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double d = L[(long long)k * n + k];
      piv = d;
      L[(long long)k * n + k] = d > 0.0 ? sqrt(d) : 0.0;
    }
    __syncthreads();
    if (!(piv > 0.0)) return;  // not SPD: the FP64 Jacobi path applies the shift
    const double lkk = L[(long long)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) L[(long long)i * n + k] /= lkk;
    __syncthreads();
    const int r = n - k - 1;
    for (long long e = threadIdx.x; e < (long long)r * r; e += blockDim.x) {
      const int i = k + 1 + (int)(e / r), j = k + 1 + (int)(e % r);
      if (j <= i) L[(long long)i * n + j] -= L[(long long)i * n + k] * L[(long long)j * n + k];
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      double s = Cd[(long long)i * n + j];
      for (int k = 0; k < i; ++k) s = fma(-L[(long long)i * n + k], Cd[(long long)k * n + j], s);
      Cd[(long long)i * n + j] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      double s = Cd[(long long)r * n + i];
      for (int k = 0; k < i; ++k) s = fma(-L[(long long)i * n + k], Cd[(long long)r * n + k], s);
      Cd[(long long)r * n + i] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    C[e] = (float)(0.5 * (Cd[e] + Cd[(long long)j * n + i]));
    U[e] = (i == j) ? 1.0f : 0.0f;
  }
  __syncthreads();
  jacobi32<false>(n, C, U, cs, pq, red);
  // X = L^-T U in FP64 (column j per thread)
  double* Xb = X + b * nn;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = n - 1; i >= 0; --i) {
      double s = (double)U[(long long)i * n + j];
      for (int k = i + 1; k < n; ++k) s = fma(-L[(long long)k * n + i], Xb[(long long)k * n + j], s);
      Xb[(long long)i * n + j] = s / L[(long long)i * n + i];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) ok[b] = 2;
}

// ---------------------------------------------------------------------------
// Stage 1 beyond the shared-memory FP32 solver (n > 128): the same
// mathematics as eigh32_fp64factor_kernel in several launches, so that the
// Cholesky and the triangular solves spread over the GPU (tiles, a warp per
// vector) instead of running as serial chains on one SM.  ok[b]: 3 after the
// Cholesky, 4 after the eigenvectors of C, 2 once X is formed.
// ---------------------------------------------------------------------------
constexpr int kVecWarps = 8;          // warps per CTA of the per-vector kernels
// the FP64 per-vector kernels (two warps per CTA, spreading the vectors over
// more SMs, ran 1.6x slower: the warps of a CTA share the triangle's rows in
// L1)
constexpr int kVec64Warps = 8;
constexpr int kMaxLargeN = 240;       // vector staging in shared memory
static_assert(kMaxLargeN <= 256, "tri_eig_kernel pairs threads j and j + 256");

// ---------------------------------------------------------------------------
// Blocked FP64 Cholesky S = L L^T over the GPU (right-looking, panels of
// kCholNb columns).  Per panel: chol_diag_kernel factors the diagonal block
// (one CTA per matrix, one barrier per column), chol_panel_kernel solves the
// rows below it against that block (a warp per row, the row's entries on the
// lanes), chol_update_kernel subtracts the panel's outer product from the
// trailing lower triangle (kCholTile x kCholTile tiles, a CTA each).  A
// matrix whose pivot is not positive drops ok to 0 and is skipped from then
// on (the FP64 Jacobi path applies the reference's shift).  Only the lower
// triangle of L is written.
// ---------------------------------------------------------------------------
constexpr int kCholNb = 32;
constexpr int kCholTile = 16;

// 1 / sqrt(x) from the FP32 estimate and two Newton steps (FP64 accuracy;
// an FP64 square root and divide cost ~10 dependent FP64 operations).
__device__ __forceinline__ double rsqrt64(double x) {
  if (!(x > 1e-30 && x < 1e30)) return 1.0 / sqrt(x);
  double y = (double)rsqrtf((float)x);
  const double h = 0.5 * x;
  y = y * fma(-h * y, y, 1.5);
  return y * fma(-h * y, y, 1.5);
}

__global__ void chol_init_kernel(int batch, int n, const double* __restrict__ A,
                                 const double* __restrict__ S, double* __restrict__ C64,
                                 double* __restrict__ L64, int* __restrict__ ok) {
  const long long tot = (long long)batch * n * n;
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long e = g; e < tot; e += (long long)gridDim.x * blockDim.x) {
    C64[e] = A[e];
    L64[e] = S[e];
  }
  for (long long b = g; b < batch; b += (long long)gridDim.x * blockDim.x) ok[b] = 3;
}

__global__ void __launch_bounds__(128) chol_diag_kernel(int n, int p0, double* __restrict__ L64,
                                                        int* __restrict__ ok) {
  const int b = blockIdx.x;
  if (ok[b] != 3) return;
  const int w = min(kCholNb, n - p0);
  __shared__ double D[kCholNb][kCholNb + 1];   // the block, updated in place (unscaled columns)
  __shared__ double Lo[kCholNb][kCholNb + 1];  // the factor's columns
  double* L = L64 + (long long)b * n * n;
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int i = e / w, j = e % w;
    D[i][j] = L[(long long)(p0 + i) * n + p0 + j];
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const double dj = D[j][j];
    if (!(dj > 0.0)) {
      if (threadIdx.x == 0) ok[b] = 0;
      return;  // dj is the same for every thread: the whole CTA leaves
    }
    const double r = rsqrt64(dj), r2 = r * r;
    // column j of the factor; the trailing block loses D[:, j] D[:, j]^T / dj
    for (int i = j + threadIdx.x; i < w; i += blockDim.x) Lo[i][j] = D[i][j] * r;
    // the trailing lower triangle, element e -> (i, l) with e = i (i + 1) / 2 + l
    const int m = w - j - 1;
    for (int e = threadIdx.x; e < m * (m + 1) / 2; e += blockDim.x) {
      int ti = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
      if ((ti + 1) * (ti + 2) / 2 <= e) ++ti;
      if (ti * (ti + 1) / 2 > e) --ti;
      const int i = j + 1 + ti, l = j + 1 + (e - ti * (ti + 1) / 2);
      D[i][l] = fma(-D[i][j] * r2, D[l][j], D[i][l]);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int i = e / w, j = e % w;
    if (j <= i) L[(long long)(p0 + i) * n + p0 + j] = Lo[i][j];
  }
}

// Rows below the panel: x L_pp^T = a, a warp per row (lane l holds a_l).
__global__ void __launch_bounds__(256) chol_panel_kernel(int n, int p0, double* __restrict__ L64,
                                                         const int* __restrict__ ok) {
  const int b = blockIdx.y;
  if (ok[b] != 3) return;
  const int w = min(kCholNb, n - p0);
  __shared__ double D[kCholNb][kCholNb + 1];
  __shared__ double rd[kCholNb];
  double* L = L64 + (long long)b * n * n;
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int i = e / w, j = e % w;
    D[i][j] = (j <= i) ? L[(long long)(p0 + i) * n + p0 + j] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < w) rd[threadIdx.x] = 1.0 / D[threadIdx.x][threadIdx.x];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = p0 + w + blockIdx.x * 8 + warp;
  if (i >= n) return;
  double a = (lane < w) ? L[(long long)i * n + p0 + lane] : 0.0;
  for (int j = 0; j < w; ++j) {
    const double xj = __shfl_sync(0xffffffffu, a, j) * rd[j];
    if (lane == j) {
      a = xj;
    } else if (lane > j && lane < w) {
      a = fma(-xj, D[lane][j], a);
    }
  }
  if (lane < w) L[(long long)i * n + p0 + lane] = a;
}

// Trailing update L_ij -= sum_l L_il L_jl (l over the panel) on the tile
// (ti, tj), tj <= ti, of the trailing lower triangle; a thread per entry.
__global__ void __launch_bounds__(kCholTile * kCholTile) chol_update_kernel(
    int n, int p0, double* __restrict__ L64, const int* __restrict__ ok) {
  const int b = blockIdx.y;
  if (ok[b] != 3) return;
  const int w = min(kCholNb, n - p0);
  const int t0 = p0 + w;
  int x = blockIdx.x, ti = 0;
  while (x > ti) {
    x -= ti + 1;
    ++ti;
  }
  const int tj = x;
  __shared__ double Pi[kCholTile][kCholNb + 1], Pj[kCholTile][kCholNb + 1];
  double* L = L64 + (long long)b * n * n;
  for (int e = threadIdx.x; e < kCholTile * w; e += blockDim.x) {
    const int r = e / w, l = e % w;
    const int ri = t0 + ti * kCholTile + r, rj = t0 + tj * kCholTile + r;
    Pi[r][l] = ri < n ? L[(long long)ri * n + p0 + l] : 0.0;
    Pj[r][l] = rj < n ? L[(long long)rj * n + p0 + l] : 0.0;
  }
  __syncthreads();
  const int r = threadIdx.x / kCholTile, c = threadIdx.x % kCholTile;
  const int i = t0 + ti * kCholTile + r, j = t0 + tj * kCholTile + c;
  if (i >= n || j > i) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int l = 0;
  for (; l + 3 < w; l += 4) {
    s0 = fma(Pi[r][l], Pj[c][l], s0);
    s1 = fma(Pi[r][l + 1], Pj[c][l + 1], s1);
    s2 = fma(Pi[r][l + 2], Pj[c][l + 2], s2);
    s3 = fma(Pi[r][l + 3], Pj[c][l + 3], s3);
  }
  for (; l < w; ++l) s0 = fma(Pi[r][l], Pj[c][l], s0);
  L[(long long)i * n + j] -= (s0 + s1) + (s2 + s3);
}

__device__ __forceinline__ double warp_sum64(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Forward substitution v <- L^-1 v for every column (rows = 0) or every row
// (rows = 1) of C64: C <- L^-1 C, then C <- C L^-T.  A warp per vector, the
// vector staged in shared memory, the dot products split over the lanes.
__global__ void __launch_bounds__(kVec64Warps * 32) tri_fwd_kernel(int n, int batch,
                                                                 const double* __restrict__ L64,
                                                                 double* __restrict__ C64,
                                                                 const int* __restrict__ ok,
                                                                 int rows) {
  __shared__ double vec[kVec64Warps][kMaxLargeN];
  __shared__ double rdiag[kVec64Warps][kMaxLargeN];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * kVec64Warps + w;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), j = (int)(gw % n);
  if (ok[b] != 3) return;
  const long long nn = (long long)n * n;
  const double* L = L64 + b * nn;
  double* Cb = C64 + b * nn;
  const long long base = rows ? (long long)j * n : j;
  const long long stride = rows ? 1 : n;
  double* v = vec[w];
  double* rd = rdiag[w];
  for (int i = lane; i < n; i += 32) {
    v[i] = Cb[base + i * stride];
    rd[i] = 1.0 / L[(long long)i * n + i];
  }
  __syncwarp();
  // column-oriented substitution: once x_i is known, the lanes update the
  // remaining entries with column i of L (no reduction on the dependent
  // chain).  Column i is read across 32 rows, whose cache lines the next 15
  // steps read again (L1 hits; rows of a transposed copy, new lines every
  // step, ran 1.9x slower, and loading the next column into registers ahead
  // of the step's __syncwarp 1.25x slower).
  for (int i = 0; i < n; ++i) {
    const double x = v[i] * rd[i];
    for (int k = i + 1 + lane; k < n; k += 32) v[k] = fma(-L[(long long)k * n + i], x, v[k]);
    __syncwarp();
    if (lane == 0) v[i] = x;
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) Cb[base + i * stride] = v[i];
}

// Jacobi of C (FP32, C in shared memory), U^T accumulated in global memory.
__global__ void __launch_bounds__(kThreads) jacobi_large_kernel(int n,
                                                                const double* __restrict__ C64,
                                                                float* __restrict__ U32,
                                                                int* __restrict__ ok) {
  const int b = blockIdx.x;
  if (ok[b] != 3) return;
  extern __shared__ float sm[];
  const long long nn = (long long)n * n;
  const int m = (n + 1) & ~1;
  float* C = sm;
  float* cs = C + nn;
  int* pq = reinterpret_cast<int*>(cs + m);
  float* red = reinterpret_cast<float*>(pq + m);
  float* U = U32 + b * nn;
  const double* Cd = C64 + b * nn;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    C[e] = (float)(0.5 * (Cd[e] + Cd[(long long)j * n + i]));
    U[e] = (i == j) ? 1.0f : 0.0f;
  }
  __syncthreads();
  jacobi32<true>(n, C, U, cs, pq, red);
  __syncthreads();
  if (threadIdx.x == 0) ok[b] = 4;
}

// ---------------------------------------------------------------------------
// FP32 eigenvectors of C beyond kMaxSmemN by tridiagonal reduction (in place
// of the one-CTA Jacobi, whose n - 1 synchronised rounds per sweep made it the
// bulk of a solve at nao 150-240):
//   tridiag_cluster_kernel: Householder reduction C = Q T Q^T over a
//     thread-block cluster (the reflectors v_k go to HV row k, d / e / tau to
//     tri);
//   tri_eig_kernel: all eigenvalues of T by Sturm counts (a counting pass,
//     then octasection) and its eigenvectors by inverse iteration with partial
//     pivoting, the vectors of a cluster (gaps below 1e-5 |T|) computed by one
//     thread in turn and orthogonalised against each other (Gram-Schmidt),
//     LAPACK stein's scheme;
//   tri_back_kernel32: u_j = H_0 ... H_{n-3} z_j over many CTAs, written as
//     row j of U^T (the layout jacobi_large_kernel produced).
// Scratch (per matrix, from the refinement's areas, idle in stage 1): HV
// (n x n floats), tri (d, e, tau, lambda: 4 n floats), and the inverse
// iteration's factors and vectors (6 n^2 floats, element i of thread j's
// array at [i n + j], so that threads stepping i together read contiguously).
// ---------------------------------------------------------------------------
__device__ inline float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Row stride of C in the Householder reduction's shared memory: rows 16-byte
// aligned.
__host__ __device__ inline int tri_ld(int n) { return (n + 3) & ~3; }



// Number of eigenvalues of T below sigma (signs of the L D L^T pivots).
__device__ inline int sturm_count32(int n, const float* d, const float* e2, float sigma,
                                    float pivmin) {
  float qv = d[0] - sigma;
  if (fabsf(qv) < pivmin) qv = -pivmin;
  int c = qv < 0.0f;
  for (int i = 1; i < n; ++i) {
    qv = d[i] - sigma - __fdividef(e2[i - 1], qv);
    if (fabsf(qv) < pivmin) qv = -pivmin;
    c += qv < 0.0f;
  }
  return c;
}

// The Householder reduction over a thread-block cluster of kCl CTAs (one
// cluster per matrix): CTA q holds rows [q R, q R + R) of C (R = ceil(n / kCl))
// in its shared memory.  Per step k two cluster barriers: (1) the owner of
// row k forms the reflector and writes v and tau into every CTA's shared
// memory (distributed shared memory); (2) every CTA forms p = tau A v for its
// rows (a warp per four rows) and writes its part of p and of v.p into every
// CTA;
// then each CTA updates its rows, A <- A - v w^T - w v^T with w = p - K v.
// The buffers written remotely alternate between two copies by step parity:
// a CTA writes step k + 1's copy only after every CTA has passed step k's
// first barrier, so nobody still reads it.  The norm of the next reflector is
// summed by its row's owner during the update.
constexpr int kCl = 8;
constexpr int kClThreads = 256;
__host__ __device__ inline int cl_rows(int n) { return (n + kCl - 1) / kCl; }

__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kClThreads)
    tridiag_cluster_kernel(int n, const double* __restrict__ C64, double* __restrict__ HVws,
                           double* __restrict__ TRIws, const int* __restrict__ ok) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const int b = blockIdx.x / kCl;
  if (ok[b] != 3) return;  // the same for the whole cluster (one matrix)
  extern __shared__ float4 smraw[];
  float* sm = reinterpret_cast<float*>(smraw);
  const int R = cl_rows(n), ld = tri_ld(n);
  float* A = sm;                  // R rows of ld floats: rows r0 .. r1 - 1 of C
  float* vbuf = A + R * ld;       // [2][n] the reflector v (absolute column index)
  float* pbuf = vbuf + 2 * n;     // [2][n] p
  float* vpbuf = pbuf + 2 * n;    // [2][kCl] the CTAs' parts of v.p
  float* scal = vpbuf + 2 * kCl;  // [2][4] tau
  float* red = scal + 8;          // 64
  const long long nn = (long long)n * n;
  float* HV = reinterpret_cast<float*>(HVws + b * nn);
  float* d = reinterpret_cast<float*>(TRIws + b * nn);
  float* e = d + n;
  float* tau = e + n;
  const double* Cd = C64 + b * nn;
  const int r0 = q * R, r1 = min(n, r0 + R);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int nw = kClThreads / 32;
  for (int r = r0 + warp; r < r1; r += nw)
    for (int c = lane; c < ld; c += 32)
      A[(r - r0) * ld + c] =
          c < n ? (float)(0.5 * (Cd[(long long)r * n + c] + Cd[(long long)c * n + r])) : 0.0f;
  // red[48]: the sum of squares of x[1 ..] of the next reflector, kept by
  // the owner of its row (summed during the previous step's update)
  if (q == 0 && warp == 0) {
    float s0 = 0.0f;
    for (int c = 2 + lane; c < n; c += 32) s0 = fmaf(A[c], A[c], s0);
    s0 = warp_sumf(s0);
    if (lane == 0) red[48] = s0;
  }
  __syncthreads();
  cluster.sync();  // every CTA of the cluster runs before any remote access
  for (int k = 0; k < n - 2; ++k) {
    const int par = k & 1;
    float* vb = vbuf + par * n;
    float* pb = pbuf + par * n;
    float* vpb = vpbuf + par * kCl;
    float* sc = scal + par * 4;
    if (q == k / R) {
      // (1) the owner of row k: the reflector of x = C[k][k+1 ..]
      const float* rk = A + (k - r0) * ld;
      if (threadIdx.x == 0) {
        const float sq = red[48];
        const float x0 = rk[k + 1];
        float alpha = x0, t = 0.0f;
        if (sq > 0.0f) {
          const float nrm = sqrtf(fmaf(x0, x0, sq));
          alpha = x0 >= 0.0f ? -nrm : nrm;
          const float u0 = x0 - alpha;
          t = 2.0f / fmaf(u0, u0, sq);
        }
        red[32] = t;
        red[33] = (t != 0.0f) ? x0 - alpha : 1.0f;
        d[k] = rk[k];
        e[k] = alpha;
        tau[k] = t;
      }
      __syncthreads();
      const float t = red[32], v0 = red[33];
      for (int c = k + 1 + threadIdx.x; c < n; c += kClThreads) {
        const float val = c == k + 1 ? v0 : rk[c];
        HV[(long long)k * n + c] = val;
#pragma unroll
        for (int t2 = 0; t2 < kCl; ++t2) cluster.map_shared_rank(vb, t2)[c] = val;
      }
      if (threadIdx.x < kCl) cluster.map_shared_rank(sc, (int)threadIdx.x)[0] = t;
    }
    cluster.sync();
    // (2) p = tau A v for this CTA's rows beyond k (four rows at a time per
    // warp, their sums and reductions interleaved), and their part of v.p
    const float t = sc[0];
    float vp = 0.0f;
    for (int rb = max(k + 1, r0) + 4 * warp; rb < r1; rb += 4 * nw) {
      float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      const float* ar = A + (rb - r0) * ld;
      for (int c = k + 1 + lane; c < n; c += 32) {
        const float vc = vb[c];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (rb + u < r1) a[u] = fmaf(ar[u * ld + c], vc, a[u]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] += __shfl_xor_sync(0xffffffffu, a[u], o);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (rb + u < r1) {
          const float pr = t * a[u];
          if (lane < kCl) cluster.map_shared_rank(pb, lane)[rb + u] = pr;
          vp = fmaf(vb[rb + u], pr, vp);
        }
      }
    }
    if (lane == 0) red[40 + warp] = vp;
    __syncthreads();
    if (threadIdx.x < kCl) {
      float s = 0.0f;
#pragma unroll
      for (int w = 0; w < nw; ++w) s += red[40 + w];
      cluster.map_shared_rank(vpb, (int)threadIdx.x)[q] = s;
    }
    cluster.sync();
    // the rank-2 update of this CTA's rows (local only)
    float qs = 0.0f;
#pragma unroll
    for (int t2 = 0; t2 < kCl; ++t2) qs += vpb[t2];
    const float K = 0.5f * t * qs;
    for (int r = max(k + 1, r0) + warp; r < r1; r += nw) {
      float* ar = A + (r - r0) * ld;
      const float vr = vb[r], wr = fmaf(-K, vr, pb[r]);
      float s2 = 0.0f;
      for (int c = k + 1 + lane; c < n; c += 32) {
        const float vc = vb[c];
        const float nv = ar[c] - fmaf(vr, fmaf(-K, vc, pb[c]), wr * vc);
        ar[c] = nv;
        if (c >= k + 3) s2 = fmaf(nv, nv, s2);
      }
      if (r == k + 1) {  // the next reflector's row: its norm for the next step
        s2 = warp_sumf(s2);
        if (lane == 0) red[48] = s2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (n - 2 >= r0 && n - 2 < r1) {
      d[n - 2] = A[(n - 2 - r0) * ld + n - 2];
      tau[n - 2] = 0.0f;
    }
    if (n - 1 >= r0 && n - 1 < r1) {
      e[n - 2] = A[(n - 1 - r0) * ld + n - 2];
      d[n - 1] = A[(n - 1 - r0) * ld + n - 1];
      e[n - 1] = 0.0f;
      tau[n - 1] = 0.0f;
    }
  }
}

// Numbers of eigenvalues of T below three shifts, their recurrences
// interleaved.
__device__ inline void sturm_count32x3(int n, const float* d, const float* e2, float s0, float s1,
                                       float s2, float pivmin, int& c0, int& c1, int& c2) {
  float q0 = d[0] - s0, q1 = d[0] - s1, q2 = d[0] - s2;
  if (fabsf(q0) < pivmin) q0 = -pivmin;
  if (fabsf(q1) < pivmin) q1 = -pivmin;
  if (fabsf(q2) < pivmin) q2 = -pivmin;
  int k0 = q0 < 0.0f, k1 = q1 < 0.0f, k2 = q2 < 0.0f;
  for (int i = 1; i < n; ++i) {
    const float di = d[i], ei = e2[i - 1];
    q0 = di - s0 - __fdividef(ei, q0);
    q1 = di - s1 - __fdividef(ei, q1);
    q2 = di - s2 - __fdividef(ei, q2);
    if (fabsf(q0) < pivmin) q0 = -pivmin;
    if (fabsf(q1) < pivmin) q1 = -pivmin;
    if (fabsf(q2) < pivmin) q2 = -pivmin;
    k0 += q0 < 0.0f;
    k1 += q1 < 0.0f;
    k2 += q2 < 0.0f;
  }
  c0 = k0;
  c1 = k1;
  c2 = k2;
}

// kSmemX: the vectors under inverse iteration live in shared memory (every
// step of a solve reads the value the previous step wrote; from global memory
// that is an L2 round trip per step), copied to INV at the end.
template <bool kSmemX>
__global__ void __launch_bounds__(kThreads) tri_eig_kernel(int n, double* __restrict__ TRIws,
                                                           double* __restrict__ INVws, int ks,
                                                           const int* __restrict__ ok) {
  const int b = blockIdx.x;
  if (ok[b] != 3) return;
  __shared__ float ds[kMaxLargeN], es[kMaxLargeN], e2[kMaxLargeN], lam[kMaxLargeN];
  const long long nn = (long long)n * n;
  const float* d = reinterpret_cast<const float*>(TRIws + b * nn);
  const float* e = d + n;
  float* W = reinterpret_cast<float*>(INVws + b * (long long)ks * nn);
  float* Lm = W;                 // multipliers
  float* U0 = W + nn;            // 1 / (U diagonal); U first and second superdiagonals
  float* U1 = W + 2 * nn;
  float* U2 = W + 3 * nn;
  float* PV = W + 4 * nn;        // 1 where rows i and i+1 were swapped
  float* Xg = W + 5 * nn;        // eigenvector of eigenvalue j in column j
  extern __shared__ float xsm[];
  float* X = kSmemX ? xsm : Xg;
  float lo = 3.0e38f, hi = -3.0e38f, nrm = 0.0f, emax = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float di = d[i], ei = (i < n - 1) ? e[i] : 0.0f, ep = i > 0 ? e[i - 1] : 0.0f;
    ds[i] = di;
    es[i] = ei;
    e2[i] = ei * ei;
    const float r = fabsf(ei) + fabsf(ep);
    lo = fminf(lo, di - r);
    hi = fmaxf(hi, di + r);
    nrm = fmaxf(nrm, fabsf(di) + r);
    emax = fmaxf(emax, ei * ei);
  }
  // block min / max
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    nrm = fmaxf(nrm, __shfl_xor_sync(0xffffffffu, nrm, o));
    emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  __shared__ float r4[4][32];
  if ((threadIdx.x & 31) == 0) {
    r4[0][threadIdx.x >> 5] = lo;
    r4[1][threadIdx.x >> 5] = hi;
    r4[2][threadIdx.x >> 5] = nrm;
    r4[3][threadIdx.x >> 5] = emax;
  }
  __syncthreads();
  lo = r4[0][0];
  hi = r4[1][0];
  nrm = r4[2][0];
  emax = r4[3][0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
    lo = fminf(lo, r4[0][w]);
    hi = fmaxf(hi, r4[1][w]);
    nrm = fmaxf(nrm, r4[2][w]);
    emax = fmaxf(emax, r4[3][w]);
  }
  nrm = fmaxf(nrm, 1e-30f);
  const float pivmin = 1.2e-38f * fmaxf(1.0f, emax);
  const float span = fmaxf(hi - lo, nrm * 1e-6f);
  lo -= 2.0f * FLT_EPSILON * span + pivmin;
  hi += 2.0f * FLT_EPSILON * span + pivmin;
  // Eigenvalue j (ascending) on threads j and j + 256 (n <= 256).  One pass of
  // counts at kThreads evenly spaced shifts (a thread each) brackets every
  // eigenvalue to (hi - lo) / kThreads; then octasection, the pair's six
  // interior shifts per pass (three each, their recurrences interleaved), to
  // an absolute width of 4 eps |T| (the shifts of the inverse iteration need
  // no more; the FP64 refinement recomputes the eigenvalues).
  __shared__ int hist[kThreads];
  __shared__ int oct[256][6];
  const float atol = 4.0f * FLT_EPSILON * nrm + pivmin;
  const float bw = (hi - lo) / (float)kThreads;
  hist[threadIdx.x] = sturm_count32(
      n, ds, e2, threadIdx.x + 1 == kThreads ? hi : fmaf(bw, (float)(threadIdx.x + 1), lo),
      pivmin);
  __syncthreads();
  const int jj = threadIdx.x & 255, q = threadIdx.x >> 8;
  float a = lo, c = hi;
  if (jj < n) {
    int l0 = 0, h0 = kThreads - 1;  // the smallest t with hist[t] > jj
    while (l0 < h0) {
      const int mid = (l0 + h0) >> 1;
      if (hist[mid] > jj) {
        h0 = mid;
      } else {
        l0 = mid + 1;
      }
    }
    a = l0 == 0 ? lo : fmaf(bw, (float)l0, lo);
    c = l0 + 1 == kThreads ? hi : fmaf(bw, (float)(l0 + 1), lo);
  }
  int passes = 0;
  for (float wd = bw; wd > atol && passes < 16; wd *= 0.125f) ++passes;
  for (int it = 0; it < passes; ++it) {
    const float h = (c - a) * (1.0f / 7.0f);
    if (jj < n) {
      int n0, n1, n2;
      sturm_count32x3(n, ds, e2, fmaf(h, (float)(1 + 3 * q), a), fmaf(h, (float)(2 + 3 * q), a),
                      fmaf(h, (float)(3 + 3 * q), a), pivmin, n0, n1, n2);
      oct[jj][3 * q] = n0;
      oct[jj][3 * q + 1] = n1;
      oct[jj][3 * q + 2] = n2;
    }
    __syncthreads();
    if (jj < n) {
      // both threads of the pair take the same sub-interval
      int mm = 1;
      while (mm <= 6 && oct[jj][mm - 1] <= jj) ++mm;
      const float na = mm == 1 ? a : fmaf(h, (float)(mm - 1), a);
      if (mm <= 6) c = fmaf(h, (float)mm, a);
      a = na;
    }
    __syncthreads();
  }
  if (jj < n && q == 0) lam[jj] = 0.5f * (a + c);
  __syncthreads();
  // inverse iteration, every eigenvector on its own thread (the members of a
  // cluster in parallel too, with shifts separated by sep in member order);
  // the clusters' vectors are orthogonalised after the iterations
  const float ctol = 1e-5f * nrm;
  const float sep = 10.0f * FLT_EPSILON * nrm;
  const float tiny = FLT_EPSILON * nrm;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    int lead = j;  // the first member of j's cluster
    while (lead > 0 && lam[lead] - lam[lead - 1] <= ctol) --lead;
    float lprev = -3.0e38f;
    for (int m2 = lead; m2 <= j; ++m2) {
      float l2 = lam[m2];
      if (m2 > lead && l2 - lprev < sep) l2 = lprev + sep;
      lprev = l2;
    }
    {
      const int mbr = j;
      const float lm = lprev;
      // T - lm I = P L U (partial pivoting); column j of the factor arrays
      float ra = ds[0] - lm, rb = n > 1 ? es[0] : 0.0f, rc = 0.0f;
      for (int i = 0; i < n - 1; ++i) {
        const float ci = es[i], an = ds[i + 1] - lm, bn = (i + 1 < n - 1) ? es[i + 1] : 0.0f;
        const long long q = (long long)i * n + j;
        if (fabsf(ci) > fabsf(ra)) {
          const float l = __fdividef(ra, ci);
          U0[q] = __frcp_rn(ci);
          U1[q] = an;
          U2[q] = bn;
          Lm[q] = l;
          PV[q] = 1.0f;
          ra = rb - l * an;
          rb = rc - l * bn;
        } else {
          const float piv = fabsf(ra) < tiny ? copysignf(tiny, ra) : ra;
          const float l = __fdividef(ci, piv);
          U0[q] = __frcp_rn(piv);
          U1[q] = rb;
          U2[q] = rc;
          Lm[q] = l;
          PV[q] = 0.0f;
          ra = an - l * rb;
          rb = bn - l * rc;
        }
        rc = 0.0f;
      }
      {
        const long long q = (long long)(n - 1) * n + j;
        U0[q] = __frcp_rn(fabsf(ra) < tiny ? copysignf(tiny, ra) : ra);
        U1[q] = 0.0f;
        U2[q] = 0.0f;
      }
      // start vector: a fixed pseudo-random pattern
      for (int i = 0; i < n; ++i)
        X[(long long)i * n + mbr] = 1.0f + 0.25f * (float)((i * 7919 + mbr * 104729) % 17) / 17.0f;
      for (int it = 0; it < 3; ++it) {
        // x <- U^-1 L^-1 P x.  The factors of kAhead steps are loaded
        // together (independent global loads, one L2 round trip per group)
        // before the dependent recurrence consumes them.
        constexpr int kAhead = 16;
        float cur = X[mbr];
        for (int i0 = 0; i0 < n - 1; i0 += kAhead) {
          float lf[kAhead], pf[kAhead];
#pragma unroll
          for (int t = 0; t < kAhead; ++t) {
            const int i = min(i0 + t, n - 2);
            lf[t] = Lm[(long long)i * n + j];
            pf[t] = PV[(long long)i * n + j];
          }
#pragma unroll
          for (int t = 0; t < kAhead; ++t) {
            const int i = i0 + t;
            if (i < n - 1) {
              // cur: entry i as updated by step i - 1 (carried in a register)
              float xi = cur, xn = X[(long long)(i + 1) * n + mbr];
              if (pf[t] != 0.0f) {
                const float tt = xi;
                xi = xn;
                xn = tt;
              }
              X[(long long)i * n + mbr] = xi;
              cur = xn - lf[t] * xi;
            }
          }
        }
        X[(long long)(n - 1) * n + mbr] = cur;
        float x1 = 0.0f, x2 = 0.0f, amax = 0.0f;
        for (int i0 = n - 1; i0 >= 0; i0 -= kAhead) {
          float f0[kAhead], f1[kAhead], f2[kAhead];
#pragma unroll
          for (int t = 0; t < kAhead; ++t) {
            const long long q = (long long)max(i0 - t, 0) * n + j;
            f0[t] = U0[q];
            f1[t] = U1[q];
            f2[t] = U2[q];
          }
#pragma unroll
          for (int t = 0; t < kAhead; ++t) {
            const int i = i0 - t;
            if (i >= 0) {
              const float xi = (X[(long long)i * n + mbr] - f1[t] * x1 - f2[t] * x2) * f0[t];
              X[(long long)i * n + mbr] = xi;
              x2 = x1;
              x1 = xi;
              amax = fmaxf(amax, fabsf(xi));
            }
          }
        }
        // scale, normalise
        const float sc = amax > 0.0f ? 1.0f / amax : 1.0f;
        for (int i = 0; i < n; ++i) X[(long long)i * n + mbr] *= sc;
        float ss = 0.0f;
        for (int i = 0; i < n; ++i) {
          const float xi = X[(long long)i * n + mbr];
          ss = fmaf(xi, xi, ss);
        }
        const float inv = ss > 0.0f ? rsqrtf(ss) : 0.0f;
        for (int i = 0; i < n; ++i) X[(long long)i * n + mbr] *= inv;
      }
    }
  }
  __syncthreads();
  // modified Gram-Schmidt inside each cluster, by its first thread in member
  // order (the vectors of a cluster span its invariant subspace to FP32
  // accuracy; the FP64 refinement and its Rayleigh-Ritz pass resolve the
  // pairs inside it)
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    if (j > 0 && lam[j] - lam[j - 1] <= ctol) continue;
    int end = j;
    while (end + 1 < n && lam[end + 1] - lam[end] <= ctol) ++end;
    for (int mbr = j + 1; mbr <= end; ++mbr) {
      for (int o = j; o < mbr; ++o) {
        float dot = 0.0f;
        for (int i = 0; i < n; ++i)
          dot = fmaf(X[(long long)i * n + o], X[(long long)i * n + mbr], dot);
        for (int i = 0; i < n; ++i)
          X[(long long)i * n + mbr] = fmaf(-dot, X[(long long)i * n + o], X[(long long)i * n + mbr]);
      }
      float ss = 0.0f;
      for (int i = 0; i < n; ++i) {
        const float xi = X[(long long)i * n + mbr];
        ss = fmaf(xi, xi, ss);
      }
      const float inv = ss > 0.0f ? rsqrtf(ss) : 0.0f;
      for (int i = 0; i < n; ++i) X[(long long)i * n + mbr] *= inv;
    }
  }
  if (kSmemX) {
    __syncthreads();
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) Xg[e] = X[e];
  }
}

// u_j = H_0 H_1 ... H_{n-3} z_j for the eigenvectors z_j of T (column j of
// the inverse iteration's X), a warp per vector; row j of U^T receives u_j.
__global__ void __launch_bounds__(kVecWarps * 32) tri_back_kernel32(int n, int batch,
                                                                    const double* __restrict__ HVws,
                                                                    const double* __restrict__ TRIws,
                                                                    const double* __restrict__ INVws,
                                                                    int ks,
                                                                    float* __restrict__ U32,
                                                                    const int* __restrict__ ok) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * kVecWarps + w;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), j = (int)(gw % n);
  if (ok[b] != 3) return;
  const long long nn = (long long)n * n;
  const float* HV = reinterpret_cast<const float*>(HVws + b * nn);
  const float* tau = reinterpret_cast<const float*>(TRIws + b * nn) + 2 * n;
  const float* X = reinterpret_cast<const float*>(INVws + b * (long long)ks * nn) + 5 * nn;
  // z in registers (entry lane + 32 t), the reflectors read one step ahead
  constexpr int kPer = (kMaxLargeN + 31) / 32;
  float zr[kPer], cv[kPer], nv[kPer];
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int i = lane + 32 * t;
    zr[t] = i < n ? X[(long long)i * n + j] : 0.0f;
  }
  if (n < 3) {
    float* u = U32 + b * nn + (long long)j * n;
#pragma unroll
    for (int t = 0; t < kPer; ++t)
      if (lane + 32 * t < n) u[lane + 32 * t] = zr[t];
    return;
  }
  // reflectors k (cv), k - 1 (nv) in registers, k - 2 loaded during step k
  float n2[kPer];
  float ct = tau[n - 3], nt = n >= 4 ? tau[n - 4] : 0.0f, t2 = 0.0f;
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int i = lane + 32 * t;
    cv[t] = (i > n - 3 && i < n) ? HV[(long long)(n - 3) * n + i] : 0.0f;
    nv[t] = (n >= 4 && i > n - 4 && i < n) ? HV[(long long)(n - 4) * n + i] : 0.0f;
  }
  for (int k = n - 3; k >= 0; --k) {
    if (k > 1) {
      const float* vn = HV + (long long)(k - 2) * n;
      t2 = tau[k - 2];
#pragma unroll
      for (int t = 0; t < kPer; ++t) {
        const int i = lane + 32 * t;
        n2[t] = (i > k - 2 && i < n) ? vn[i] : 0.0f;
      }
    }
    if (ct != 0.0f) {
      float a = 0.0f;
#pragma unroll
      for (int t = 0; t < kPer; ++t) a = fmaf(cv[t], zr[t], a);
      a = ct * warp_sumf(a);
#pragma unroll
      for (int t = 0; t < kPer; ++t) zr[t] = fmaf(-a, cv[t], zr[t]);
    }
    ct = nt;
    nt = t2;
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      cv[t] = nv[t];
      nv[t] = n2[t];
    }
  }
  float* u = U32 + b * nn + (long long)j * n;
#pragma unroll
  for (int t = 0; t < kPer; ++t)
    if (lane + 32 * t < n) u[lane + 32 * t] = zr[t];
}

__global__ void stage_done_kernel(int batch, int* __restrict__ ok, int from, int to) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < batch; b += gridDim.x * blockDim.x)
    if (ok[b] == from) ok[b] = to;
}

// X[:, j] = L^-T u_j (backward substitution, FP64), u_j = row j of U^T.
__global__ void __launch_bounds__(kVec64Warps * 32) tri_back_kernel(int n, int batch,
                                                                  const double* __restrict__ L64,
                                                                  const float* __restrict__ U32,
                                                                  double* __restrict__ X,
                                                                  const int* __restrict__ ok) {
  __shared__ double vec[kVec64Warps][kMaxLargeN];
  __shared__ double rdiag[kVec64Warps][kMaxLargeN];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * kVec64Warps + w;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), j = (int)(gw % n);
  if (ok[b] != 4) return;
  const long long nn = (long long)n * n;
  const double* L = L64 + b * nn;
  const float* u = U32 + b * nn + (long long)j * n;
  double* v = vec[w];
  double* rd = rdiag[w];
  for (int i = lane; i < n; i += 32) {
    v[i] = (double)u[i];
    rd[i] = 1.0 / L[(long long)i * n + i];
  }
  __syncwarp();
  // L^T x = u from the bottom: once x_i is known, the lanes update the
  // entries above it with row i of L (contiguous)
  for (int i = n - 1; i >= 0; --i) {
    const double x = v[i] * rd[i];
    const double* Li = L + (long long)i * n;
    for (int k = lane; k < i; k += 32) v[k] = fma(-Li[k], x, v[k]);
    __syncwarp();
    if (lane == 0) v[i] = x;
    __syncwarp();
  }
  double* Xb = X + b * nn;
  for (int i = lane; i < n; i += 32) Xb[(long long)i * n + j] = v[i];
}

__global__ void large_done_kernel(int batch, int* __restrict__ ok) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < batch; b += gridDim.x * blockDim.x)
    if (ok[b] == 4) ok[b] = 2;
}

// Batched split-K FP64 GEMM partials: P[b][kc] = op(A_b)[:, kc chunk] B_b[kc chunk, :]
// (n x n, op = transpose with kTA).  grid (tiles, tiles, batch * ksplit).
// Early acceptance: a step whose check passes (X accurate to ~1e-7) sets
// kDoneNext; that step's update X' = X + X E still runs (it brings X to the
// FP64 floor, as the last step does), then kDone replaces kDoneNext and the
// remaining steps skip the matrix (their update X' = X + X E copies X).
constexpr int kDone = 16;
constexpr int kDoneNext = 32;

template <bool kTA>
__global__ void __launch_bounds__(kGThreads) gemm_part_kernel(int n, int ksplit,
                                                              const double* __restrict__ A,
                                                              const double* __restrict__ B,
                                                              double* __restrict__ P,
                                                              const int* __restrict__ skip) {
  __shared__ double As[kKC][kT + 1];
  __shared__ double Bs[kKC][kT + 1];
  const long long nn = (long long)n * n;
  const int b = blockIdx.z / ksplit, kc = blockIdx.z % ksplit;
  if (skip && (skip[b] & kDone)) return;
  const int r0 = blockIdx.y * kT, c0 = blockIdx.x * kT;
  const int k0 = kc * kKC;
  const double* Ab = A + b * nn;
  const double* Bb = B + b * nn;
  for (int e = threadIdx.x; e < kKC * kT; e += kGThreads) {
    const int k = e / kT, c = e % kT;
    const int kk = k0 + k;
    double a = 0.0, v = 0.0;
    if (kk < n) {
      if (r0 + c < n) a = kTA ? Ab[(long long)kk * n + r0 + c] : Ab[(long long)(r0 + c) * n + kk];
      if (c0 + c < n) v = Bb[(long long)kk * n + c0 + c];
    }
    As[k][c] = a;
    Bs[k][c] = v;
  }
  __syncthreads();
  // 16 x 16 threads, 2 x 2 outputs each
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[2][2] = {};
#pragma unroll
  for (int k = 0; k < kKC; ++k) {
    const double a0 = As[k][ty * 2], a1 = As[k][ty * 2 + 1];
    const double b0 = Bs[k][tx * 2], b1 = Bs[k][tx * 2 + 1];
    acc[0][0] = fma(a0, b0, acc[0][0]);
    acc[0][1] = fma(a0, b1, acc[0][1]);
    acc[1][0] = fma(a1, b0, acc[1][0]);
    acc[1][1] = fma(a1, b1, acc[1][1]);
  }
  double* Pb = P + ((long long)b * ksplit + kc) * nn;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int r = r0 + ty * 2 + i, c = c0 + tx * 2 + j;
      if (r < n && c < n) Pb[(long long)r * n + c] = acc[i][j];
    }
}

// C_b = base + sign * sum_kc P[b][kc] (fixed order).  base: kIdentity -> I,
// else the matrix `base` (may be null: 0).
__global__ void gemm_sum_kernel(int batch, int n, int ksplit, const double* __restrict__ P,
                                const double* base, bool identity, double sign, double* C,
                                const int* __restrict__ skip) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < batch * nn;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / nn, o = e % nn;
    if (skip && (skip[b] & kDone)) {
      if (base && !identity) C[e] = base[e];
      continue;
    }
    double s = 0.0;
    for (int kc = 0; kc < ksplit; ++kc) s += P[(b * ksplit + kc) * nn + o];
    double v = identity ? ((o / n == o % n) ? 1.0 : 0.0) : (base ? base[e] : 0.0);
    C[e] = fma(sign, s, v);
  }
}

// As = (A + A^T)/2, Ss = (S + S^T)/2 for every matrix of the batch.
__global__ void sym_kernel(int batch, int n, const double* __restrict__ A,
                           const double* __restrict__ S, double* __restrict__ As,
                           double* __restrict__ Ss) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < batch * nn;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / nn, o = e % nn;
    const long long t = b * nn + (o % n) * n + o / n;
    As[e] = 0.5 * (A[e] + A[t]);
    Ss[e] = 0.5 * (S[e] + S[t]);
  }
}

// kDoneNext -> kDone once the accepting step's update has run.
__global__ void done_next_kernel(int batch, int* __restrict__ ok) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch && (ok[b] & kDoneNext)) ok[b] = (ok[b] & ~kDoneNext) | kDone;
}

// Refinement step, part 1: per 8-row block of every matrix (grid (row blocks,
// matrices), a warp per row) lambda_i = t_ii / (1 - r_ii) and the block's
// partial sums of |T - D|_F^2, |A|_F^2 and |R|_F^2 (in `part`, 4 doubles per
// block, a fixed summation order).
__global__ void __launch_bounds__(256) refine_partials_kernel(int n, const double* __restrict__ A,
                                                              const double* __restrict__ R,
                                                              const double* __restrict__ T,
                                                              double* __restrict__ lam,
                                                              double* __restrict__ part,
                                                              const int* __restrict__ ok) {
  __shared__ double red[3][8];
  const int b = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (ok[b] & kDone) return;
  const int i = blockIdx.x * 8 + warp;
  const long long nn = (long long)n * n;
  double od = 0.0, an = 0.0, rn = 0.0;
  if (i < n) {
    const double* tr = T + b * nn + (long long)i * n;
    const double* ar = A + b * nn + (long long)i * n;
    const double* rr = R + b * nn + (long long)i * n;
    const double li = tr[i] / (1.0 - rr[i]);
    if (lane == 0) lam[(long long)b * n + i] = li;
    for (int j = lane; j < n; j += 32) {
      const double d = tr[j] - (i == j ? li : 0.0);
      od = fma(d, d, od);
      an = fma(ar[j], ar[j], an);
      rn = fma(rr[j], rr[j], rn);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    od += __shfl_xor_sync(0xffffffffu, od, o);
    an += __shfl_xor_sync(0xffffffffu, an, o);
    rn += __shfl_xor_sync(0xffffffffu, rn, o);
  }
  if (lane == 0) {
    red[0][warp] = od;
    red[1][warp] = an;
    red[2][warp] = rn;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[threadIdx.x][w];
    part[((long long)b * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = t;
  }
}

// The pairwise check of the last two steps: per block the largest
// t_ij^2 / (d + sqrt(d^2 + t_ij^2)), d = |lambda_j - lambda_i| / 2 (slot 3).
__global__ void __launch_bounds__(256) refine_pairs_kernel(int n, const double* __restrict__ T,
                                                           const double* __restrict__ lam,
                                                           double* __restrict__ part,
                                                           const int* __restrict__ ok) {
  __shared__ double red[8];
  const int b = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (ok[b] & kDone) return;
  const int i = blockIdx.x * 8 + warp;
  const long long nn = (long long)n * n;
  double pe = 0.0;
  if (i < n) {
    const double* tr = T + b * nn + (long long)i * n;
    const double* lb = lam + (long long)b * n;
    const double li = lb[i];
    for (int j = lane; j < n; j += 32) {
      if (j == i) continue;
      const double d = 0.5 * fabs(lb[j] - li), t2 = tr[j] * tr[j];
      const double q = d + sqrt(fma(d, d, t2));
      if (q > 0.0) pe = fmax(pe, t2 / q);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pe = fmax(pe, __shfl_xor_sync(0xffffffffu, pe, o));
  if (lane == 0) red[warp] = pe;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < 8; ++w) m = fmax(m, red[w]);
    part[((long long)b * gridDim.x + blockIdx.x) * 4 + 3] = m;
  }
}

// Refinement step, part 2 (a thread per matrix): Ogita and Aishima's
// threshold delta (delta[b]) from the partial sums and the acceptance checks.
__global__ void refine_final_kernel(int batch, int blocks, const double* __restrict__ part,
                                    double* __restrict__ delta_out, int* __restrict__ ok,
                                    int check) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch || (ok[b] & kDone)) return;
  double od = 0.0, an = 0.0, rn = 0.0, pe = 0.0;
  for (int k = 0; k < blocks; ++k) {
    const double* q = part + ((long long)b * blocks + k) * 4;
    od += q[0];
    an += q[1];
    rn += q[2];
    if (check >= 2) pe = fmax(pe, q[3]);
  }
  // Frobenius norms bound the 2-norms of Ogita and Aishima's threshold
  delta_out[b] = 2.0 * (sqrt(od) + sqrt(an) * sqrt(rn));
  // last step: the X it refines must already be accurate to ~1e-7 (it is
  // unless S is too ill-conditioned for the FP32 solve), so that this step
  // reaches the FP64 floor; otherwise hand the matrix to the FP64 path.
  // Checks 2 and 3 also bound, for every pair, how far the diagonal of T is
  // from the eigenvalues of its 2 x 2 block (an unresolved near-degenerate
  // pair leaves both off by ~T_ij^2 / gap although |T - D|_F is small).
  // Check 1: this step decides; 2 and 3: the last two steps, either passing
  // suffices (at the FP64 floor of an ill-conditioned S, |R| fluctuates from
  // step to step by orders of magnitude); 4: a step before those, where
  // passing ends the matrix's refinement after this step's update.
  if (check && ok[b] != 0) {
    const bool pass = rn <= 1e-14 && od <= 1e-14 * an && (check < 2 || pe <= 1e-12 * sqrt(an));
    if (check == 1) {
      if (!pass) ok[b] = 0;
    } else if (check == 4) {
      if (pass) ok[b] |= kDoneNext;
    } else if (check == 2) {
      if (!pass) ok[b] |= 8;
    } else if (pass) {
      ok[b] &= ~8;
    } else if (ok[b] & 8) {
      ok[b] = 0;
    }
  }
}

// Refinement step, part 2: the correction E over the GPU (a warp per row,
// grid (rows / 8, matrices)).
__global__ void __launch_bounds__(256) refine_e_kernel(int n, const double* __restrict__ R,
                                                       const double* __restrict__ T,
                                                       const double* __restrict__ lam,
                                                       const double* __restrict__ delta,
                                                       double* __restrict__ E,
                                                       const int* __restrict__ ok) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= n || (ok[b] & kDone)) return;
  const long long nn = (long long)n * n;
  const double* rr = R + b * nn + (long long)i * n;
  const double* tr = T + b * nn + (long long)i * n;
  double* er = E + b * nn + (long long)i * n;
  const double* lb = lam + (long long)b * n;
  const double li = lb[i], dl = delta[b];
  for (int j = lane; j < n; j += 32) {
    double v;
    if (i == j) {
      v = 0.5 * rr[j];
    } else {
      const double gap = lb[j] - li;
      v = (fabs(gap) > dl) ? (tr[j] + lb[j] * rr[j]) / gap : 0.5 * rr[j];
    }
    er[j] = v;
  }
}

// Rayleigh-Ritz on strongly mixed pairs: T = X^T A X of a nearly
// S-orthonormal X; the pairs (i, j) with |t_ij| > 2^-10 |t_ii - t_jj| (a mixing
// angle above ~1e-3) are rotated by FP64 Jacobi rotations (three sweeps over
// the pair list, in a fixed order) applied to T and to the columns of X.  The
// FP32 start cannot resolve pairs closer than ~1e-7 |C|; their first-order
// corrections would be O(1), outside the refinement's convergence region (and
// pairs inside its cluster threshold are never separated at all).  At most
// kMaxPairs pairs (else nothing is done).
constexpr int kMaxPairs = 512;

__global__ void __launch_bounds__(kThreads) cluster_jacobi_kernel(int n, double* __restrict__ T,
                                                                  double* __restrict__ X,
                                                                  const int* __restrict__ ok) {
  const int b = blockIdx.x;
  if (!ok[b]) return;
  __shared__ int cnt[kThreads];
  __shared__ int pi[kMaxPairs], pj[kMaxPairs];
  __shared__ double rot[2];
  __shared__ int npair;
  const long long nn = (long long)n * n;
  double* Tb = T + b * nn;
  double* Xb = X + b * nn;
  // pair list in (i, j) order: counts per row, prefix, fill (n <= kThreads).
  // The test |t_ij| > 2^-10 |t_ii - t_jj| runs on the bit patterns (the
  // magnitudes of doubles order as their bits; 2^-10 lowers the exponent),
  // with one FP64 subtraction per pair.
  __shared__ double diag[kThreads];
  for (int i = threadIdx.x; i < n; i += blockDim.x) diag[i] = Tb[(long long)i * n + i];
  __syncthreads();
  auto mixed = [&](int i, int j) {
    const long long a = __double_as_longlong(Tb[(long long)i * n + j]) & 0x7fffffffffffffffLL;
    const long long d = __double_as_longlong(diag[i] - diag[j]) & 0x7fffffffffffffffLL;
    constexpr long long kShift = 10LL << 52;
    return a > (d > kShift ? d - kShift : 0LL);
  };
  const int i0 = threadIdx.x;
  int c = 0;
  if (i0 < n)
    for (int j = i0 + 1; j < n; ++j) c += mixed(i0, j);
  cnt[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const int v = cnt[t];
      cnt[t] = acc;
      acc += v;
    }
    npair = acc;
  }
  __syncthreads();
  if (npair > kMaxPairs || npair == 0) return;
  if (i0 < n) {
    int q = cnt[i0];
    for (int j = i0 + 1; j < n; ++j)
      if (mixed(i0, j)) {
        pi[q] = i0;
        pj[q] = j;
        ++q;
      }
  }
  __syncthreads();
  const int np = npair;
  for (int sweep = 0; sweep < 3; ++sweep) {
    for (int q = 0; q < np; ++q) {
      const int i = pi[q], j = pj[q];
      if (threadIdx.x == 0) {
        // the angle in FP32 from the FP64 difference (the pass only has to
        // bring the pair into the refinement's convergence region), then
        // (c, s) normalised in FP64 so that the rotation stays orthogonal:
        // a dozen dependent FP64 operations instead of two divides and two
        // square roots on the serial path
        const double tij = Tb[(long long)i * n + j];
        double cc = 1.0, ss = 0.0;
        const float tf = (float)tij;
        if (tf != 0.0f && isfinite(tf)) {
          const float tau = (float)(Tb[(long long)j * n + j] - Tb[(long long)i * n + i]) /
                            (2.0f * tf);
          const float t = (tau >= 0.0f ? 1.0f : -1.0f) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.0f)));
          const double c0 = (double)rsqrtf(fmaf(t, t, 1.0f)), s0 = (double)t * c0;
          const double r = rsqrt64(fma(c0, c0, s0 * s0));
          cc = c0 * r;
          ss = s0 * r;
        }
        rot[0] = cc;
        rot[1] = ss;
      }
      __syncthreads();
      const double cc = rot[0], ss = rot[1];
      if (ss != 0.0) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {  // columns i, j of T and X
          const double ti = Tb[(long long)k * n + i], tj = Tb[(long long)k * n + j];
          Tb[(long long)k * n + i] = cc * ti - ss * tj;
          Tb[(long long)k * n + j] = ss * ti + cc * tj;
          const double xi = Xb[(long long)k * n + i], xj = Xb[(long long)k * n + j];
          Xb[(long long)k * n + i] = cc * xi - ss * xj;
          Xb[(long long)k * n + j] = ss * xi + cc * xj;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += blockDim.x) {  // rows i, j of T
          const double ti = Tb[(long long)i * n + k], tj = Tb[(long long)j * n + k];
          Tb[(long long)i * n + k] = cc * ti - ss * tj;
          Tb[(long long)j * n + k] = ss * ti + cc * tj;
        }
      }
      __syncthreads();
    }
  }
}

// Ascending (stable) order: w[b][rank_i] = lambda_i, V[b][:, rank_i] = X[:, i].
__global__ void sort_out_kernel(int n, const double* __restrict__ lam,
                                const double* __restrict__ X, const int* __restrict__ ok,
                                double* __restrict__ w, double* __restrict__ V,
                                int32_t* __restrict__ status) {
  extern __shared__ long long key[];  // n order-preserving integer keys, then n ranks
  int* rank = reinterpret_cast<int*>(key + n);
  const int b = blockIdx.x;
  if (!ok[b]) return;
  const long long nn = (long long)n * n;
  const double* lb = lam + (long long)b * n;
  // the integer image of a double that orders as the double does (negative
  // values: all bits but the sign flipped), so that the ranks need no FP64
  // compares
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long kb = __double_as_longlong(lb[i]);
    key[i] = kb >= 0 ? kb : kb ^ 0x7fffffffffffffffLL;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long ki = key[i];
    int r = 0;
    for (int j = 0; j < n; ++j) r += (key[j] < ki) || (key[j] == ki && j < i);
    rank[i] = r;
    w[(long long)b * n + r] = lb[i];
  }
  __syncthreads();
  // a warp per row: coalesced reads, writes permuted within the row
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int i = warp; i < n; i += nw) {
    const double* xr = X + b * nn + (long long)i * n;
    double* vr = V + b * nn + (long long)i * n;
    for (int j = lane; j < n; j += 32) vr[rank[j]] = xr[j];
  }
  if (threadIdx.x == 0 && status) status[b] = 0;
}

}  // namespace qex_mp

namespace qex_mp_host {

using namespace qex_mp;

constexpr int kMaxSmemN = 128;  // eigh32_kernel: 3 n^2 FP32 matrices in shared memory
constexpr int kMaxN = 240;      // beyond kMaxSmemN: C alone in shared memory (checked at launch)
static_assert(kMaxN <= kMaxLargeN, "per-vector kernels stage up to kMaxLargeN entries");

int ksplit_of(int n) { return (n + kKC - 1) / kKC; }

// Doubles of the mixed-precision area per matrix: As, Ss, X, X', T, R, E
// (7 n^2), split-K partials (ksplit n^2), lambda (n), the FP64 factor and
// transformed matrix of the FP64-factor stage (2 n^2), one spare; beyond
// kMaxSmemN also U^T in FP32 (n^2 floats).
long long area_doubles(int n) {
  const long long nn = (long long)n * n;
  // U^T in FP32 is reserved at every size: the path of a size is selectable
  // ... then delta and the refinement's partial sums (4 per 8-row block)
  return (9 + ksplit_of(n)) * nn + n + 1 + (nn + 1) / 2 + 1 + 4 * ((n + 7) / 8);
}

// Path per matrix size: 0 the default (shared-memory FP32 solve up to
// kMaxSmemN, the FP64 factor and tridiagonal stage beyond), 1 the
// shared-memory solve, 2 the FP64 factor and tridiagonal stage.
std::atomic<int> g_path[kMaxN + 1];

size_t smem_factor64(int n) {
  const int m = (n + 1) & ~1;
  return sizeof(float) * (2 * (size_t)n * n + 2 * (size_t)m + 33);
}

size_t smem_factor64_large(int n) {
  const int m = (n + 1) & ~1;
  return sizeof(float) * ((size_t)n * n + 2 * (size_t)m + 33);
}

size_t smem_tridiag_cluster(int n) {
  return sizeof(float) * ((size_t)cl_rows(n) * tri_ld(n) + 4 * (size_t)n + 2 * kCl + 8 + 64);
}

size_t smem32(int n) {
  const int m = (n + 1) & ~1;
  return sizeof(float) * (3 * (size_t)n * n + 2 * (size_t)m + 35);
}

void gemm(cudaStream_t s, int batch, int n, bool ta, const double* A, const double* B, double* P,
          const double* base, bool identity, double sign, double* C,
          const int* skip = nullptr) {
  const int ks = ksplit_of(n);
  const int tiles = (n + kT - 1) / kT;
  const dim3 grid(tiles, tiles, (unsigned)(batch * ks));
  if (ta) {
    gemm_part_kernel<true><<<grid, kGThreads, 0, s>>>(n, ks, A, B, P, skip);
  } else {
    gemm_part_kernel<false><<<grid, kGThreads, 0, s>>>(n, ks, A, B, P, skip);
  }
  const long long work = (long long)batch * n * n;
  const int blocks = (int)((work + 255) / 256 < 4096 ? (work + 255) / 256 : 4096);
  gemm_sum_kernel<<<blocks, 256, 0, s>>>(batch, n, ks, P, base, identity, sign, C, skip);
}

}  // namespace qex_mp_host

// Host entry used by qex_td_gen_eigh: runs the mixed-precision solver on the
// batch and leaves ok[b] = 0 for matrices that need the FP64 path.  Returns
// false when n is beyond the solver (n > 240, or C does not fit in shared
// memory; then nothing was launched).
bool qex_mp_gen_eigh(int batch, int n, const double* A, const double* S, double* w, double* V,
                     int32_t* status, double* area, int* ok_out, cudaStream_t s) {
  using namespace qex_mp_host;
  if (n > kMaxN) return false;
  const int path = g_path[n].load(std::memory_order_relaxed);
  // the tridiagonal path needs n >= 8 (its reduction leaves a 2 x 2 block and
  // splits the rows over kCl CTAs); smaller matrices always take the
  // shared-memory solve
  const bool large =
      n >= kCl && (path == 2 || n > kMaxSmemN) && !(path == 1 && n <= kMaxSmemN);
  int max_optin = 0;
  if (large) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem_factor64_large(n) + 64 > (size_t)max_optin) return false;  // + static shared
    if (smem_tridiag_cluster(n) + 64 > (size_t)max_optin) return false;
  }
  const long long nn = (long long)n * n;
  const long long per = (long long)batch * nn;
  double* As = area;
  double* Ss = As + per;
  double* X = Ss + per;
  double* X2 = X + per;
  double* T = X2 + per;
  double* R = T + per;
  double* E = R + per;
  double* P = E + per;
  double* lam = P + (long long)ksplit_of(n) * per;
  double* L64 = lam + (long long)batch * n;
  double* C64 = L64 + per;
  // one double per matrix after the FP32 U^T area (within the area's spare)
  double* dlt = reinterpret_cast<double*>(reinterpret_cast<float*>(C64 + per) + ((per + 1) & ~1LL));
  double* part = dlt + batch;  // 4 per 8-row block of every matrix
  int* ok = ok_out;
  const int eb = (int)((per + 255) / 256 < 4096 ? (per + 255) / 256 : 4096);
  sym_kernel<<<eb, 256, 0, s>>>(batch, n, A, S, As, Ss);
  if (!large) {
    const size_t sm = smem32(n);
    cudaFuncSetAttribute(eigh32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    eigh32_kernel<<<batch, kThreads, sm, s>>>(n, As, Ss, X, ok);
    // overlaps too ill-conditioned for the FP32 Cholesky: FP64 factor, FP32 Jacobi
    const size_t sm64 = smem_factor64(n);
    cudaFuncSetAttribute(eigh32_fp64factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm64);
    eigh32_fp64factor_kernel<<<batch, kThreads, sm64, s>>>(n, As, Ss, X, L64, C64, ok);
  } else {
    // every matrix: FP64 factor and transformation, FP32 Jacobi with C in
    // shared memory and U^T in global memory, FP64 back-transformation
    float* U32 = reinterpret_cast<float*>(C64 + per);
    chol_init_kernel<<<eb, 256, 0, s>>>(batch, n, As, Ss, C64, L64, ok);  // ok <- 3
    for (int p0 = 0; p0 < n; p0 += kCholNb) {
      chol_diag_kernel<<<batch, 128, 0, s>>>(n, p0, L64, ok);
      const int rows = n - p0 - min(kCholNb, n - p0);
      if (rows > 0) {
        chol_panel_kernel<<<dim3((unsigned)((rows + 7) / 8), (unsigned)batch), 256, 0, s>>>(
            n, p0, L64, ok);
        const int T = (rows + kCholTile - 1) / kCholTile;
        chol_update_kernel<<<dim3((unsigned)(T * (T + 1) / 2), (unsigned)batch),
                             kCholTile * kCholTile, 0, s>>>(n, p0, L64, ok);
      }
    }
    const long long vecs = (long long)batch * n;
    const unsigned vb = (unsigned)((vecs + kVecWarps - 1) / kVecWarps);
    const unsigned vb64 = (unsigned)((vecs + kVec64Warps - 1) / kVec64Warps);
    tri_fwd_kernel<<<vb64, kVec64Warps * 32, 0, s>>>(n, batch, L64, C64, ok, 0);  // C <- L^-1 C
    tri_fwd_kernel<<<vb64, kVec64Warps * 32, 0, s>>>(n, batch, L64, C64, ok, 1);  // C <- C L^-T
    // eigenvectors of C in FP32: Householder tridiagonalisation, bisection and
    // inverse iteration, back-transformation (scratch: T, R and P, idle until
    // the refinement)
    const size_t smt = smem_tridiag_cluster(n);
    cudaFuncSetAttribute(tridiag_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smt);
    tridiag_cluster_kernel<<<batch * kCl, kClThreads, smt, s>>>(n, C64, T, R, ok);
    const int ks = ksplit_of(n);
    const size_t smx = sizeof(float) * (size_t)n * n;
    if (smx + 16384 <= (size_t)max_optin &&  // + the kernel's static shared memory
        cudaFuncSetAttribute(tri_eig_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smx) == cudaSuccess) {
      tri_eig_kernel<true><<<batch, kThreads, smx, s>>>(n, R, P, ks, ok);
    } else {
      tri_eig_kernel<false><<<batch, kThreads, 0, s>>>(n, R, P, ks, ok);
    }
    tri_back_kernel32<<<vb, kVecWarps * 32, 0, s>>>(n, batch, T, R, P, ks, U32, ok);
    stage_done_kernel<<<(batch + 255) / 256, 256, 0, s>>>(batch, ok, 3, 4);
    tri_back_kernel<<<vb64, kVec64Warps * 32, 0, s>>>(n, batch, L64, U32, X, ok);
    large_done_kernel<<<(batch + 255) / 256, 256, 0, s>>>(batch, ok);
  }
  // four steps; beyond the shared-memory solver up to six, with a
  // Rayleigh-Ritz pass on strongly mixed pairs after the first, the third
  // and fourth accepting X early when it passes the check (after that step's
  // update the remaining steps skip the matrix; accepting after the second
  // left near-degenerate pairs mixed at ~1e-7, 3e-7 Ha in an SCF energy), and
  // the last two checked (either passing suffices)
  const int steps = large ? kRefineSteps + 2 : kRefineSteps;
  const int* skip = large ? ok : nullptr;
  for (int it = 0; it < steps; ++it) {
    if (large && it == 1) {
      gemm(s, batch, n, false, As, X, P, nullptr, false, 1.0, T);  // T = A X
      gemm(s, batch, n, true, X, T, P, nullptr, false, 1.0, E);    // E <- X^T A X
      cluster_jacobi_kernel<<<batch, kThreads, 0, s>>>(n, E, X, ok);
    }
    gemm(s, batch, n, false, Ss, X, P, nullptr, false, 1.0, T, skip);   // T = S X
    gemm(s, batch, n, true, X, T, P, nullptr, true, -1.0, R, skip);     // R = I - X^T S X
    gemm(s, batch, n, false, As, X, P, nullptr, false, 1.0, T, skip);   // T = A X
    gemm(s, batch, n, true, X, T, P, nullptr, false, 1.0, E, skip);     // E <- X^T A X
    // move X^T A X into T and build the correction in E
    cudaMemcpyAsync(T, E, sizeof(double) * per, cudaMemcpyDeviceToDevice, s);
    const int check = !large ? (it == steps - 1 ? 1 : 0)
                             : (it == steps - 2 ? 2
                                                : (it == steps - 1 ? 3 : (it >= 2 ? 4 : 0)));
    const dim3 rgrid((unsigned)((n + 7) / 8), (unsigned)batch);
    refine_partials_kernel<<<rgrid, 256, 0, s>>>(n, As, R, T, lam, part, ok);
    if (check >= 2) refine_pairs_kernel<<<rgrid, 256, 0, s>>>(n, T, lam, part, ok);
    refine_final_kernel<<<(batch + 127) / 128, 128, 0, s>>>(batch, (n + 7) / 8, part, dlt, ok,
                                                            check);
    refine_e_kernel<<<dim3((unsigned)((n + 7) / 8), (unsigned)batch), 256, 0, s>>>(n, R, T, lam, dlt,
                                                                                  E, ok);
    gemm(s, batch, n, false, X, E, P, X, false, 1.0, X2, skip);         // X' = X + X E
    if (large && it >= 2) done_next_kernel<<<(batch + 255) / 256, 256, 0, s>>>(batch, ok);
    double* t = X;
    X = X2;
    X2 = t;
  }
  sort_out_kernel<<<batch, 256, (sizeof(long long) + sizeof(int)) * n, s>>>(n, lam, X, ok, w, V,
                                                                             status);
  return true;
}

// Selects the path of matrices of size n (see g_path); false when n is beyond
// the mixed-precision solver or path is unknown.
bool qex_mp_set_path(int n, int path) {
  if (n < 1 || n > qex_mp_host::kMaxN || path < 0 || path > 2) return false;
  qex_mp_host::g_path[n].store(path, std::memory_order_relaxed);
  return true;
}

// Doubles of mixed-precision workspace per matrix (0 when n is beyond it).
long long qex_mp_area_doubles(int n) {
  return n <= qex_mp_host::kMaxN ? qex_mp_host::area_doubles(n) : 0;
}
