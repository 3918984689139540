// Warp-level evaluation of the global-local convolutional KSR functional for
// one molecule (qedft/models/classical/global_ksr_model.py:32-80, built from
// jax_dft neural_xc: global_conv_block, two bias-free width-3 convolutions with
// swish, a width-1 convolution, the negativity transform -swish, and the
// self-interaction layer).  Produces eps over the grid, the partial E_xc sum
// of this lane, and optionally the potential
//   local convention:     v = eps + J^T n       (jax_dft, (dE/dn)/dx)
//   amplitude convention: v = dx J^T 1          (qedft scf.py:53-76)
// with J = d eps / d n.
//
// Layout: one lane per grid point.  The grid is walked in chunks of 32 lanes
// that own 24 points each; the 4 halo points either side cover the reach of
// the two width-3 layers, forward and backward, so both passes stay in
// registers and warp shuffles.  The 15 exponential global convolutions and the
// self-interaction Hartree term are exponentially weighted sums
//   sum_j x_j r^|i-j|,  r = exp(-dx / w),
// computed as a left and a right warp scan per chunk plus carries: left
// carries run with the sweep; right carries come from a reverse pre-pass over
// the chunks (forward) or are applied after the sweep through a recursion over
// the chunks (backward: the transposed convolution of the per-point
// gradients).  All network arithmetic is FP32; sums over points are FP64.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "const_slots.cuh"
#include "ks1d_common.cuh"
#include "qex_ks1d.h"

namespace qex {

constexpr int kKsrMaxC = QEX_KSR_CHANNELS;  // largest supported channel count
constexpr int kKsrOwn = 24;                  // points owned by one 32-lane chunk
constexpr int kKsrHalo = 4;                  // halo either side
// the self-interaction layer uses jax_dft exponential_coulomb's defaults
constexpr double kKsrSiAmplitude = 1.071295;
constexpr double kKsrSiKappa = 1.0 / 2.385345;

// Packed parameter offsets for C channels (C global filters = C local filters):
// W1 (3, C, C), W2 (3, C, C), W3 (C), eta (C - 1), self-interaction width.
template <int C>
struct KsrLayout {
  static constexpr int kScans = C;  // C - 1 global widths + the self-interaction Hartree
  static constexpr int kW1 = 0, kW2 = 3 * C * C, kW3 = 6 * C * C, kEta = 6 * C * C + C;
  static constexpr int kWidth = 6 * C * C + 2 * C - 1;
  static constexpr int kParams = 6 * C * C + 2 * C;
};

// The network of a launch is staged in constant memory (const_slots.cuh) so
// that every weight is a warp-uniform operand of the FMA that uses it.
constexpr int kKsrSlots = 4;
constexpr int kKsrSlotFloat4 = (6 * kKsrMaxC * kKsrMaxC + 2 * kKsrMaxC) / 4;
static __constant__ float4 c_ksr_w[kKsrSlots][kKsrSlotFloat4];

__host__ __device__ inline int ksr_chunks(int n) { return (n + kKsrOwn - 1) / kKsrOwn; }

// per-warp FP32 scratch for up to kKsrMaxC channels: power tables (2 x C x 32),
// per-scan constants and carries (6 x C), right-carry tables (2 x C x chunks)
__host__ __device__ inline size_t ksr_scratch_floats(int nmax) {
  return (size_t)2 * kKsrMaxC * kWarp + 6 * kKsrMaxC + (size_t)2 * kKsrMaxC * ksr_chunks(nmax);
}

struct KsrScratch {
  float* pf;  // [C][32]: r^(lane + 1)
  float* pr;  // [C][32]: r^(32 - lane)
  float* r;   // [C] decay per point
  float* q;   // [C] dx / w
  float* cf;  // [C] forward coefficients
  float* cb;  // [C] backward coefficients
  float* lc;  // [C] forward left carries
  float* lb;  // [C] backward left carries
  float* rc;  // [chunks][C] forward right carries R(p0 + 32)
  float* rl;  // [chunks][C] backward local suffix sums, then right carries
};

template <int C>
__device__ inline KsrScratch ksr_carve(float* base, int nchunks) {
  KsrScratch s;
  s.pf = base;
  s.pr = s.pf + C * kWarp;
  s.r = s.pr + C * kWarp;
  s.q = s.r + C;
  s.cf = s.q + C;
  s.cb = s.cf + C;
  s.lc = s.cb + C;
  s.lb = s.lc + C;
  s.rc = s.lb + C;
  s.rl = s.rc + C * nchunks;
  return s;
}

// S_l = x_l + r S_{l-1} over the lanes (Hillis-Steele with decay powers)
__device__ __forceinline__ float ksr_scan_up(float x, float r, int lane) {
  #pragma unroll
  for (int d = 1; d < kWarp; d <<= 1) {
    const float t = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x = fmaf(r, t, x);
    r *= r;
  }
  return x;
}

// S_l = x_l + r S_{l+1}
__device__ __forceinline__ float ksr_scan_down(float x, float r, int lane) {
  #pragma unroll
  for (int d = 1; d < kWarp; d <<= 1) {
    const float t = __shfl_down_sync(kFull, x, d);
    if (lane + d < kWarp) x = fmaf(r, t, x);
    r *= r;
  }
  return x;
}

__device__ __forceinline__ float ksr_sigmoid(float x) { return __fdividef(1.0f, 1.0f + __expf(-x)); }

// z[o] += sum_t v(p + t - 1) W[t][c][o] for one input channel c (Wc = &W[0][c][0])
template <int C>
__device__ __forceinline__ void ksr_conv_in(float (&z)[C], float v, const float4* Wc) {
  const float vm = __shfl_up_sync(kFull, v, 1);
  const float vp = __shfl_down_sync(kFull, v, 1);
  #pragma unroll
  for (int q = 0; q < C / 4; ++q) {
    const float4 a = *(Wc + q);
    const float4 b = *(Wc + C * C / 4 + q);
    const float4 c = *(Wc + C * C / 2 + q);
    z[4 * q + 0] = fmaf(vm, a.x, fmaf(v, b.x, fmaf(vp, c.x, z[4 * q + 0])));
    z[4 * q + 1] = fmaf(vm, a.y, fmaf(v, b.y, fmaf(vp, c.y, z[4 * q + 1])));
    z[4 * q + 2] = fmaf(vm, a.z, fmaf(v, b.z, fmaf(vp, c.z, z[4 * q + 2])));
    z[4 * q + 3] = fmaf(vm, a.w, fmaf(v, b.w, fmaf(vp, c.w, z[4 * q + 3])));
  }
}

// sum_o d[o] W[t][c][o] (Wtc = &W[t][c][0])
template <int C>
__device__ __forceinline__ float ksr_dot_row(const float (&d)[C], const float4* Wtc) {
  float s = 0.0f;
  #pragma unroll
  for (int q = 0; q < C / 4; ++q) {
    const float4 a = *(Wtc + q);
    s = fmaf(d[4 * q + 0], a.x, s);
    s = fmaf(d[4 * q + 1], a.y, s);
    s = fmaf(d[4 * q + 2], a.z, s);
    s = fmaf(d[4 * q + 3], a.w, s);
  }
  return s;
}

// Per-molecule constants and tables.  Returns beta and writes d beta / d I.
template <int C>
__device__ inline double ksr_setup(const float* __restrict__ w, double lo, double hi, int N,
                                   double dx, const double* n, const KsrScratch& S, int nchunks,
                                   double& dbeta, int lane) {
  using Ly = KsrLayout<C>;
  double part = 0.0;
  #pragma unroll 1
  for (int i = lane; i < N; i += kWarp) part += n[i];
  const double integral = warp_sum(part) * dx;
  const double width = (double)w[Ly::kWidth];
  const double u = (integral - 1.0) / width;
  const double beta = exp(-u * u);
  dbeta = beta * (-2.0 * u / width);
  if (lane < Ly::kScans) {
    double q, cf, cb;
    if (lane < Ly::kScans - 1) {
      const double wj = lo + (hi - lo) / (1.0 + exp(-(double)w[Ly::kEta + lane]));
      q = dx / wj;
      cf = dx / (2.0 * wj);
      cb = cf;
    } else {
      q = kKsrSiKappa * dx;
      cf = -0.5 * kKsrSiAmplitude * dx;
      cb = cf * beta;
    }
    S.q[lane] = (float)q;
    S.r[lane] = (float)exp(-q);
    S.cf[lane] = (float)cf;
    S.cb[lane] = (float)cb;
    S.lc[lane] = 0.0f;
    S.lb[lane] = 0.0f;
    S.rc[(nchunks - 1) * Ly::kScans + lane] = 0.0f;
  }
  __syncwarp();
  #pragma unroll 1
  for (int j = 0; j < Ly::kScans; ++j) {
    const float q = S.q[j];
    S.pf[j * kWarp + lane] = expf(-q * (float)(lane + 1));
    S.pr[j * kWarp + lane] = expf(-q * (float)(kWarp - lane));
  }
  __syncwarp();
  return beta;
}

// kGroup scans are staged and run together (independent shuffle chains that
// overlap); more groups need more registers, so the SCF kernel, which calls
// this under its register cap, uses 1 and the standalone evaluator 4.
template <int C, bool kWantV, int kGroup>
__device__ __noinline__ double ksr_eval(const float* __restrict__ w, int slot, double lo, double hi,
                                        int N, double dx, const double* n, bool local,
                                        double* vout, double* frec, float* scratch, int lane) {
  using Ly = KsrLayout<C>;
  const int K = ksr_chunks(N);
  const KsrScratch S = ksr_carve<C>(scratch, K);
  double dbeta;
  const double beta = ksr_setup<C>(w, lo, hi, N, dx, n, S, K, dbeta, lane);
  const float fb = (float)beta, f1b = (float)(1.0 - beta);
  const float4* W1 = c_ksr_w[slot] + Ly::kW1 / 4;
  const float4* W2 = c_ksr_w[slot] + Ly::kW2 / 4;
  const float4* W3 = c_ksr_w[slot] + Ly::kW3 / 4;

  // right carries of the forward scans: chunk k needs R(p0_k + 32), which is
  // lane 32 - kKsrOwn of chunk k + 1
  #pragma unroll 1
  for (int k = K - 1; k >= 1; --k) {
    const int p = k * kKsrOwn - kKsrHalo + lane;
    const float x = (p >= 0 && p < N) ? (float)n[p] : 0.0f;
    // kGroup channels per pass, staged in registers: their scan chains overlap
    #pragma unroll 1
    for (int j0 = 0; j0 < Ly::kScans; j0 += kGroup) {
      float R[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const int j = j0 + i;
        R[i] = S.pr[j * kWarp + lane] * S.rc[k * Ly::kScans + j];
      }
      float r[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) r[i] = S.r[j0 + i];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) R[i] += ksr_scan_down(x, r[i], lane);
      float nxt[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) nxt[i] = __shfl_sync(kFull, R[i], kWarp - kKsrOwn);
      if (lane == 0) {
        #pragma unroll
        for (int i = 0; i < kGroup; ++i) S.rc[(k - 1) * Ly::kScans + j0 + i] = nxt[i];
      }
    }
    __syncwarp();
  }

  double e = 0.0, sdb = 0.0;
  #pragma unroll 1
  for (int k = 0; k < K; ++k) {
    const int p = k * kKsrOwn - kKsrHalo + lane;
    const bool in = (p >= 0 && p < N);
    const double n64 = in ? n[p] : 0.0;
    const float x = (float)n64;

    // ---- forward: channels feed the first convolution as they are made
    float z1[C];
    #pragma unroll
    for (int o = 0; o < C; ++o) z1[o] = 0.0f;
    ksr_conv_in(z1, x, W1);  // channel 0: the density
    float h = 0.0f;
    // kGroup scans per pass, their tables and carries staged in registers so
    // their shuffle chains overlap
    #pragma unroll 1
    for (int j0 = 0; j0 < Ly::kScans; j0 += kGroup) {
      float L[kGroup], R[kGroup], r[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const int j = j0 + i;
        r[i] = S.r[j];
        L[i] = S.pf[j * kWarp + lane] * S.lc[j];
        R[i] = S.pr[j * kWarp + lane] * S.rc[k * Ly::kScans + j];
      }
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        L[i] += ksr_scan_up(x, r[i], lane);
        R[i] += ksr_scan_down(x, r[i], lane);
      }
      float carry[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) carry[i] = __shfl_sync(kFull, L[i], kKsrOwn - 1);
      if (lane == 0) {
        #pragma unroll
        for (int i = 0; i < kGroup; ++i) S.lc[j0 + i] = carry[i];
      }
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const int j = j0 + i;
        const float G = S.cf[j] * (L[i] + R[i] - x);
        if (j < Ly::kScans - 1) {
          ksr_conv_in(z1, in ? G : 0.0f, W1 + (j + 1) * (C / 4));
        } else {
          h = G;
        }
      }
    }
    __syncwarp();
    float a[C];
    #pragma unroll
    for (int o = 0; o < C; ++o) a[o] = in ? z1[o] * ksr_sigmoid(z1[o]) : 0.0f;
    // second convolution in the output-stationary form: per tap t, this
    // lane's contribution Q_t[o] = sum_c a[c] W2[t][c][o] moves to lane - t + 1
    float z2[C];
    #pragma unroll
    for (int o = 0; o < C; ++o) z2[o] = 0.0f;
    #pragma unroll 1
    for (int t = 0; t < 3; ++t) {
      float qv[C];
      #pragma unroll
      for (int o = 0; o < C; ++o) qv[o] = 0.0f;
      #pragma unroll
      for (int c = 0; c < C; ++c) {
        const float4* Wr = W2 + (t * C + c) * (C / 4);
        #pragma unroll
        for (int q = 0; q < C / 4; ++q) {
          const float4 wv = *(Wr + q);
          qv[4 * q + 0] = fmaf(a[c], wv.x, qv[4 * q + 0]);
          qv[4 * q + 1] = fmaf(a[c], wv.y, qv[4 * q + 1]);
          qv[4 * q + 2] = fmaf(a[c], wv.z, qv[4 * q + 2]);
          qv[4 * q + 3] = fmaf(a[c], wv.w, qv[4 * q + 3]);
        }
      }
      // z2 at lane l takes Q_t from the lane of point l + t - 1
      #pragma unroll
      for (int o = 0; o < C; ++o) z2[o] += __shfl_sync(kFull, qv[o], lane + t - 1);
    }
    float y = 0.0f;
    #pragma unroll
    for (int q = 0; q < C / 4; ++q) {
      const float4 wv = *(W3 + q);
      a[4 * q + 0] = z2[4 * q + 0] * ksr_sigmoid(z2[4 * q + 0]);
      a[4 * q + 1] = z2[4 * q + 1] * ksr_sigmoid(z2[4 * q + 1]);
      a[4 * q + 2] = z2[4 * q + 2] * ksr_sigmoid(z2[4 * q + 2]);
      a[4 * q + 3] = z2[4 * q + 3] * ksr_sigmoid(z2[4 * q + 3]);
      y = fmaf(a[4 * q + 0], wv.x, y);
      y = fmaf(a[4 * q + 1], wv.y, y);
      y = fmaf(a[4 * q + 2], wv.z, y);
      y = fmaf(a[4 * q + 3], wv.w, y);
    }
    const float sy = ksr_sigmoid(y);
    const float o = -y * sy;
    const float eps = fmaf(fb, h, f1b * o);
    const bool owned = in && lane >= kKsrHalo && lane < kKsrHalo + kKsrOwn;
    if (owned) {
      e += local ? (double)eps * n64 : (double)eps;
      if (frec) frec[p] = (double)eps;
    }
    if (!kWantV) continue;

    // ---- backward with cotangent g (n, or 1), injected where the forward
    // is valid (lanes 2..29)
    const bool v2 = in && lane >= 2 && lane < kWarp - 2;
    const float g = v2 ? (local ? x : 1.0f) : 0.0f;
    const float dy = -f1b * g * sy * fmaf(y, 1.0f - sy, 1.0f);
    float dz[C];
    #pragma unroll
    for (int q = 0; q < C / 4; ++q) {
      const float4 wv = *(W3 + q);
      const float w4[4] = {wv.x, wv.y, wv.z, wv.w};
      #pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float zz = z2[4 * q + i];
        const float s = ksr_sigmoid(zz);
        dz[4 * q + i] = dy * w4[i] * s * fmaf(zz, 1.0f - s, 1.0f);
      }
    }
    // da1[c] = sum_t sum_o dz2(p + 1 - t)[o] W2[t][c][o]
    float da[C];
    #pragma unroll
    for (int c = 0; c < C; ++c) da[c] = 0.0f;
    #pragma unroll 1
    for (int t = 0; t < 3; ++t) {
      float sv[C];
      #pragma unroll
      for (int o = 0; o < C; ++o) sv[o] = __shfl_sync(kFull, dz[o], lane + 1 - t);
      #pragma unroll
      for (int c = 0; c < C; ++c) da[c] += ksr_dot_row(sv, W2 + (t * C + c) * (C / 4));
    }
    #pragma unroll
    for (int c = 0; c < C; ++c) {
      const float s = ksr_sigmoid(z1[c]);
      dz[c] = in ? da[c] * s * fmaf(z1[c], 1.0f - s, 1.0f) : 0.0f;
    }
    // input-channel gradients df_c(p) = sum_t P_t(p + 1 - t), P_t = sum_o dz1[o] W1[t][c][o];
    // channel 0 is the density itself, channels 1..15 go through the
    // transposed global convolutions, and scan 15 carries the self-interaction
    // Hartree term of the cotangent
    float dn;
    {
      const float P0 = ksr_dot_row(dz, W1);
      const float P1 = ksr_dot_row(dz, W1 + C * C / 4);
      const float P2 = ksr_dot_row(dz, W1 + C * C / 2);
      dn = __shfl_down_sync(kFull, P0, 1) + P1 + __shfl_up_sync(kFull, P2, 1);
    }
    const int lo_idx = lane >= kKsrHalo ? lane - kKsrHalo : 0;
    #pragma unroll 1
    for (int j0 = 0; j0 < Ly::kScans; j0 += kGroup) {
      float u[kGroup], L[kGroup], T[kGroup], r[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const int j = j0 + i;
        r[i] = S.r[j];
        L[i] = S.pf[j * kWarp + lo_idx] * S.lb[j];
        if (j < Ly::kScans - 1) {
          const float4* Wc = W1 + (j + 1) * (C / 4);
          const float P0 = ksr_dot_row(dz, Wc);
          const float P1 = ksr_dot_row(dz, Wc + C * C / 4);
          const float P2 = ksr_dot_row(dz, Wc + C * C / 2);
          u[i] = __shfl_down_sync(kFull, P0, 1) + P1 + __shfl_up_sync(kFull, P2, 1);
        } else {
          u[i] = g;
        }
        u[i] = owned ? u[i] : 0.0f;
      }
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        L[i] += ksr_scan_up(u[i], r[i], lane);
        T[i] = ksr_scan_down(u[i], r[i], lane);
      }
      float carry[kGroup], loc[kGroup];
      #pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        carry[i] = __shfl_sync(kFull, L[i], kKsrHalo + kKsrOwn - 1);
        loc[i] = __shfl_sync(kFull, T[i], kKsrHalo);
        dn = fmaf(S.cb[j0 + i], L[i] + T[i] - u[i], dn);
      }
      if (lane == 0) {
        #pragma unroll
        for (int i = 0; i < kGroup; ++i) {
          S.lb[j0 + i] = carry[i];
          S.rl[k * Ly::kScans + j0 + i] = loc[i];
        }
      }
    }
    __syncwarp();
    if (owned) {
      sdb += (double)g * ((double)h - (double)o);
      vout[p] = (local ? (double)eps : 0.0) + (double)dn;
    }
  }
  if (kWantV) {
    // right carries of the transposed scans: Rin_k = R'(first point after
    // chunk k's owned range) = loc_{k+1} + r^24 Rin_{k+1}
    if (lane < Ly::kScans) {
      const float rS = S.pf[lane * kWarp + kKsrOwn - 1];
      float rin = 0.0f;
      #pragma unroll 1
      for (int k = K - 1; k >= 0; --k) {
        const float loc = S.rl[k * Ly::kScans + lane];
        S.rl[k * Ly::kScans + lane] = rin;
        rin = fmaf(rS, rin, loc);
      }
    }
    const double dterm = warp_sum(sdb) * dbeta * dx;
    __syncwarp();
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      const int k = i / kKsrOwn;
      const int m = i - k * kKsrOwn + kKsrHalo + (kWarp - kKsrHalo - kKsrOwn);  // r^(28 - l)
      float acc = 0.0f;
      #pragma unroll 4
      for (int j = 0; j < Ly::kScans; ++j)
        acc = fmaf(S.cb[j] * S.pr[j * kWarp + m], S.rl[k * Ly::kScans + j], acc);
      const double v = vout[i] + (double)acc + dterm;
      vout[i] = local ? v : dx * v;
    }
    __syncwarp();
  }
  return e;
}

// Host: the slot table of this translation unit's KSR constant array.
namespace {
ConstSlots<kKsrSlots> g_ksr_const;

// Stages nfloats floats of the device buffer `params` for a launch on `stream`.
inline ConstStage<kKsrSlots> ksr_stage(const float* params, int nfloats, cudaStream_t stream) {
  return ConstStage<kKsrSlots>(g_ksr_const, (const void*)&c_ksr_w, sizeof(c_ksr_w[0]), params,
                               sizeof(float) * (size_t)nfloats, cudaMemcpyDeviceToDevice, stream);
}
}  // namespace
}  // namespace qex
