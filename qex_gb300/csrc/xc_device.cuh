// Device-side exchange-correlation building blocks shared by the 1D kernels.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "qex_ks1d.h"
#include "ks1d_common.cuh"

namespace qex {

// Window-MLP weights, carried by value in the kernel parameters and copied
// into shared memory by each warp.  (Constant-memory slots, which pay off for
// the larger KSR network, measured 2% slower here.)
struct MlpParams {
  float w1[QEX_MLP_WINDOW * QEX_MLP_HIDDEN];
  float b1[QEX_MLP_HIDDEN];
  float w2[QEX_MLP_HIDDEN * QEX_MLP_HIDDEN];
  float b2[QEX_MLP_HIDDEN];
  float w3[QEX_MLP_HIDDEN];
  float b3;
  float norm_inv;
};

// Exponential-Coulomb uniform-gas LDA (jax_dft xc.py, called at
// qedft/train/od/eval.py:79; published fit of Baker et al., PRB 91, 235141).
// Constants hoisted per call site; kDeriv adds d eps / d n.  Divisions are
// Newton reciprocals (ks1d_common.cuh) wherever the argument is inside the
// FP32 normal range, the exact operations otherwise (density tails).
struct LdaConsts {
  double pik;   // pi / kappa
  double ax;    // A / (2 pi)
  double ma_pi; // -A / pi
  double c3;    // pi kappa^2 / A
};

__device__ inline LdaConsts lda_consts(double A, double kappa) {
  const double pi = 3.141592653589793;
  return LdaConsts{pi / kappa, A / (2.0 * pi), -A / pi, pi * kappa * kappa / A};
}

// IEEE division kept out of line (rarely taken fallbacks stay small).
__device__ __noinline__ inline double div_exact(double a, double b) { return a / b; }

template <bool kDeriv>
__device__ inline void lda_exp_coulomb(double n, const LdaConsts& c, double& eps,
                                       double& deps_dn) {
  const double y = c.pik * n;
  double ex, dex = 0.0;
  if (y > 1e-15) {
    const double l = log1p(y * y);
    const double iy = (y > 1e-30 && y < 1e30) ? recip_nr(y) : div_exact(1.0, y);
    ex = c.ax * fma(l, iy, -2.0 * atan(y));
    if (kDeriv) dex = -c.ax * l * iy * iy;
  } else {
    ex = c.ax * (-y + y * y * y / 6.0);
    if (kDeriv) dex = c.ax * (-1.0 + 0.5 * y * y);
  }
  double ec, dec = 0.0;
  if (y > 0.0) {
    const double sy = sqrt(y);
    // P(s), s = sqrt(y): 2 - 1.00077 s + 6.26099 s^2 - 11.9041 s^3 + 9.62614 s^4
    //                    - 1.48334 s^5 + c3 s^6
    const double P =
        fma(sy, fma(sy, fma(sy, fma(sy, fma(sy, fma(sy, c.c3, -1.48334), 9.62614), -11.9041),
                            6.26099),
                    -1.00077),
            2.0);
    const double iP = (P > 1e-30 && P < 1e30) ? recip_nr(P) : div_exact(1.0, P);
    ec = c.ma_pi * y * iP;
    if (kDeriv) {
      // dP/dy = (dP/ds) / (2 s)
      const double dPds =
          fma(sy,
              fma(sy, fma(sy, fma(sy, fma(sy, 6.0 * c.c3, -5.0 * 1.48334), 4.0 * 9.62614),
                          -3.0 * 11.9041),
                  2.0 * 6.26099),
              -1.00077);
      const double isy = (sy > 1e-30 && sy < 1e30) ? recip_nr(sy) : div_exact(1.0, sy);
      const double dP = 0.5 * dPds * isy;
      dec = c.ma_pi * (P - y * dP) * iP * iP;
    }
  } else {
    ec = 0.0;
    if (kDeriv) dec = c.ma_pi / 2.0;
  }
  eps = ex + ec;
  if (kDeriv) deps_dn = (dex + dec) * c.pik;
}

// The window MLP runs in FP32 (the configuration's network arithmetic) or, as
// a checking mode, in FP64 (weights then read from global memory).
__device__ inline float mlp_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ inline double mlp_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ inline float mlp_sigmoid(float z) {
  return __fdividef(1.0f, 1.0f + __expf(-z));  // 0 when exp(-z) overflows: silu -> 0
}
__device__ inline double mlp_sigmoid(double z) { return 1.0 / (1.0 + exp(-z)); }

template <typename T>
__device__ inline T silu_d(T z, T& d) {
  const T s = mlp_sigmoid(z);
  d = s * (T(1) + z * (T(1) - s));
  return z * s;
}

// Window-MLP forward (and optionally input gradient) for one point.
// W: the 577 weights in shared memory, 16-byte aligned, in MlpParams order
// (w1 [17][16], b1, w2 [16][16], b2, w3, b3); every weight read is a
// broadcast 16-byte load of (part of) one weight row, issued next to its use.
// win: the 17 window inputs (already divided by the normalization), read from
// shared memory with stride `wstride`.  scr: per-lane shared scratch of 32
// floats at stride `ss` (hidden activations and derivatives).  With kGrad,
// scr[k * ss] (k < 17) receives d eps / d input_k on return.
constexpr int kMlpFloats = 580;  // 577 weights padded to 16 bytes
constexpr int kMlpScratch = 32;  // h1, then d1 (overwritten in place by g1)


__device__ inline void mlp_load4(const float* W, int off, float& a, float& b, float& c, float& d) {
  float4 r = *reinterpret_cast<const float4*>(W + off);
  a = r.x;
  b = r.y;
  c = r.z;
  d = r.w;
}

// FP64 weights (global memory, 16-byte aligned)
__device__ inline void mlp_load4(const double* W, int off, double& a, double& b, double& c,
                                 double& d) {
  const double2 r0 = __ldg(reinterpret_cast<const double2*>(W + off));
  const double2 r1 = __ldg(reinterpret_cast<const double2*>(W + off + 2));
  a = r0.x;
  b = r0.y;
  c = r1.x;
  d = r1.y;
}

template <bool kGrad, typename T>
__device__ inline T mlp_point(const T* W, const T* win, int wstride, T* scr, int ss) {
  T z[QEX_MLP_HIDDEN];
#pragma unroll
  for (int q = 0; q < 4; ++q) mlp_load4(W, 272 + 4 * q, z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
#pragma unroll 1
  for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
    const T x = win[k * wstride];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T a, b, c, d;
      mlp_load4(W, 16 * k + 4 * q, a, b, c, d);
      z[4 * q] = mlp_fma(x, a, z[4 * q]);
      z[4 * q + 1] = mlp_fma(x, b, z[4 * q + 1]);
      z[4 * q + 2] = mlp_fma(x, c, z[4 * q + 2]);
      z[4 * q + 3] = mlp_fma(x, d, z[4 * q + 3]);
    }
  }
#pragma unroll
  for (int h = 0; h < QEX_MLP_HIDDEN; ++h) {
    T d;
    scr[h * ss] = silu_d(z[h], d);  // h1
    scr[(16 + h) * ss] = d;         // d1
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) mlp_load4(W, 544 + 4 * q, z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
#pragma unroll 1
  for (int k = 0; k < QEX_MLP_HIDDEN; ++k) {
    const T x = scr[k * ss];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T a, b, c, d;
      mlp_load4(W, 288 + 16 * k + 4 * q, a, b, c, d);
      z[4 * q] = mlp_fma(x, a, z[4 * q]);
      z[4 * q + 1] = mlp_fma(x, b, z[4 * q + 1]);
      z[4 * q + 2] = mlp_fma(x, c, z[4 * q + 2]);
      z[4 * q + 3] = mlp_fma(x, d, z[4 * q + 3]);
    }
  }
  T out = W[576];
  T g2[QEX_MLP_HIDDEN];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    T w3[4];
    mlp_load4(W, 560 + 4 * q, w3[0], w3[1], w3[2], w3[3]);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      T d;
      T a = silu_d(z[4 * q + e], d);
      out = mlp_fma(a, w3[e], out);
      g2[4 * q + e] = w3[e] * d;
    }
  }
  if (kGrad) {
#pragma unroll 1
    for (int k = 0; k < QEX_MLP_HIDDEN; ++k) {
      T a = T(0);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        T r0, r1, r2, r3;
        mlp_load4(W, 288 + 16 * k + 4 * q, r0, r1, r2, r3);
        a = mlp_fma(r0, g2[4 * q], a);
        a = mlp_fma(r1, g2[4 * q + 1], a);
        a = mlp_fma(r2, g2[4 * q + 2], a);
        a = mlp_fma(r3, g2[4 * q + 3], a);
      }
      scr[(16 + k) * ss] = a * scr[(16 + k) * ss];  // g1 = (W2 g2) * d1, over d1
    }
    T g1[QEX_MLP_HIDDEN];
#pragma unroll
    for (int h = 0; h < QEX_MLP_HIDDEN; ++h) g1[h] = scr[(16 + h) * ss];
#pragma unroll 1
    for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
      T a = T(0);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        T r0, r1, r2, r3;
        mlp_load4(W, 16 * k + 4 * q, r0, r1, r2, r3);
        a = mlp_fma(r0, g1[4 * q], a);
        a = mlp_fma(r1, g1[4 * q + 1], a);
        a = mlp_fma(r2, g1[4 * q + 2], a);
        a = mlp_fma(r3, g1[4 * q + 3], a);
      }
      scr[k * ss] = a;  // h1 / d1 slots are dead here
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Adjoint support: dual-number forward (value y and tangent dy along the input
// direction t) followed by the reverse pass of  ybar * y + dybar * dy.
// Per-lane shared records (stride rs) for the parameter-gradient reduction:
//   [0,17) x   [17,34) t   [34,50) zbar1  [50,66) dzbar1  [66,82) h1
//   [82,98) dh1  [98,114) zbar2  [114,130) dzbar2  [130,146) w3bar  [146] ybar
//   [147,164) xbar (d/dx of the objective, not a parameter record)
// Returns dy.
constexpr int kMlpRec = 164;

template <typename T>
__device__ inline T silu_dd(T z, T& d1, T& d2) {
  const T s = mlp_sigmoid(z);
  d1 = s * (T(1) + z * (T(1) - s));
  d2 = s * (T(1) - s) * (T(2) + z * (T(1) - T(2) * s));
  return z * s;
}

template <typename T>
__device__ inline T mlp_dual_reverse(const T* W, const T* win, int wstride, const T* twin,
                                     int tstride, T ybar, T dybar, T* rec, int rs) {
  T z[QEX_MLP_HIDDEN], dz[QEX_MLP_HIDDEN];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    mlp_load4(W, 272 + 4 * q, z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
    dz[4 * q] = dz[4 * q + 1] = dz[4 * q + 2] = dz[4 * q + 3] = T(0);
  }
#pragma unroll 1
  for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
    const T x = win[k * wstride], t = twin[k * tstride];
    rec[k * rs] = x;
    rec[(17 + k) * rs] = t;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T a, b, c, d;
      mlp_load4(W, 16 * k + 4 * q, a, b, c, d);
      z[4 * q] = mlp_fma(x, a, z[4 * q]);
      z[4 * q + 1] = mlp_fma(x, b, z[4 * q + 1]);
      z[4 * q + 2] = mlp_fma(x, c, z[4 * q + 2]);
      z[4 * q + 3] = mlp_fma(x, d, z[4 * q + 3]);
      dz[4 * q] = mlp_fma(t, a, dz[4 * q]);
      dz[4 * q + 1] = mlp_fma(t, b, dz[4 * q + 1]);
      dz[4 * q + 2] = mlp_fma(t, c, dz[4 * q + 2]);
      dz[4 * q + 3] = mlp_fma(t, d, dz[4 * q + 3]);
    }
  }
  // layer 1 activations: h1, dh1 to records; keep s1', s1'' * dz1 for the reverse
  T s1p[QEX_MLP_HIDDEN], s1q[QEX_MLP_HIDDEN];
#pragma unroll
  for (int h = 0; h < QEX_MLP_HIDDEN; ++h) {
    T d1, d2;
    const T a = silu_dd(z[h], d1, d2);
    rec[(66 + h) * rs] = a;
    rec[(82 + h) * rs] = d1 * dz[h];
    s1p[h] = d1;
    s1q[h] = d2 * dz[h];
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    mlp_load4(W, 544 + 4 * q, z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
    dz[4 * q] = dz[4 * q + 1] = dz[4 * q + 2] = dz[4 * q + 3] = T(0);
  }
#pragma unroll 1
  for (int k = 0; k < QEX_MLP_HIDDEN; ++k) {
    const T x = rec[(66 + k) * rs], t = rec[(82 + k) * rs];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T a, b, c, d;
      mlp_load4(W, 288 + 16 * k + 4 * q, a, b, c, d);
      z[4 * q] = mlp_fma(x, a, z[4 * q]);
      z[4 * q + 1] = mlp_fma(x, b, z[4 * q + 1]);
      z[4 * q + 2] = mlp_fma(x, c, z[4 * q + 2]);
      z[4 * q + 3] = mlp_fma(x, d, z[4 * q + 3]);
      dz[4 * q] = mlp_fma(t, a, dz[4 * q]);
      dz[4 * q + 1] = mlp_fma(t, b, dz[4 * q + 1]);
      dz[4 * q + 2] = mlp_fma(t, c, dz[4 * q + 2]);
      dz[4 * q + 3] = mlp_fma(t, d, dz[4 * q + 3]);
    }
  }
  // layer 2, output, and the reverse of the output layer
  T dy = T(0);
  T zb2[QEX_MLP_HIDDEN], dzb2[QEX_MLP_HIDDEN];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    T w3[4];
    mlp_load4(W, 560 + 4 * q, w3[0], w3[1], w3[2], w3[3]);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int h = 4 * q + e;
      T d1, d2;
      const T h2 = silu_dd(z[h], d1, d2);
      const T dh2 = d1 * dz[h];
      dy = mlp_fma(w3[e], dh2, dy);
      rec[(130 + h) * rs] = ybar * h2 + dybar * dh2;  // w3bar
      const T hb2 = ybar * w3[e], dhb2 = dybar * w3[e];
      zb2[h] = hb2 * d1 + dhb2 * d2 * dz[h];
      dzb2[h] = dhb2 * d1;
      rec[(98 + h) * rs] = zb2[h];
      rec[(114 + h) * rs] = dzb2[h];
    }
  }
  rec[146 * rs] = ybar;
  // reverse of layer 2: hbar1 = W2 zbar2, dhbar1 = W2 dzbar2
#pragma unroll 1
  for (int k = 0; k < QEX_MLP_HIDDEN; ++k) {
    T hb = T(0), dhb = T(0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T r0, r1, r2, r3;
      mlp_load4(W, 288 + 16 * k + 4 * q, r0, r1, r2, r3);
      hb = mlp_fma(r0, zb2[4 * q], hb);
      hb = mlp_fma(r1, zb2[4 * q + 1], hb);
      hb = mlp_fma(r2, zb2[4 * q + 2], hb);
      hb = mlp_fma(r3, zb2[4 * q + 3], hb);
      dhb = mlp_fma(r0, dzb2[4 * q], dhb);
      dhb = mlp_fma(r1, dzb2[4 * q + 1], dhb);
      dhb = mlp_fma(r2, dzb2[4 * q + 2], dhb);
      dhb = mlp_fma(r3, dzb2[4 * q + 3], dhb);
    }
    // zbar1 = hbar1 s1' + dhbar1 s1'' dz1 ; dzbar1 = dhbar1 s1'
    rec[(34 + k) * rs] = hb;   // temporarily hbar1
    rec[(50 + k) * rs] = dhb;  // temporarily dhbar1
  }
  T zb1[QEX_MLP_HIDDEN];
#pragma unroll
  for (int h = 0; h < QEX_MLP_HIDDEN; ++h) {
    const T hb = rec[(34 + h) * rs], dhb = rec[(50 + h) * rs];
    zb1[h] = hb * s1p[h] + dhb * s1q[h];
    rec[(34 + h) * rs] = zb1[h];
    rec[(50 + h) * rs] = dhb * s1p[h];
  }
  // xbar = W1 zbar1
#pragma unroll 1
  for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
    T a = T(0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T r0, r1, r2, r3;
      mlp_load4(W, 16 * k + 4 * q, r0, r1, r2, r3);
      a = mlp_fma(r0, zb1[4 * q], a);
      a = mlp_fma(r1, zb1[4 * q + 1], a);
      a = mlp_fma(r2, zb1[4 * q + 2], a);
      a = mlp_fma(r3, zb1[4 * q + 3], a);
    }
    rec[(147 + k) * rs] = a;
  }
  return dy;
}

// Parameter gradient of one round: sum over the 32 lanes' records, parameter p
// handled by lane p % 32 into acc[p / 32] (FP64 accumulators).
template <typename T>
__device__ inline void mlp_param_grad_round(const T* recbase, int lane, double* acc) {
  // recbase: records of lane l at recbase[f * 32 + l]
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const int pidx = lane + 32 * q;
    if (pidx >= 577) break;
    T s = T(0);
    if (pidx < 272) {
      const int a = pidx >> 4, h = pidx & 15;
      for (int l = 0; l < 32; ++l)
        s += recbase[a * 32 + l] * recbase[(34 + h) * 32 + l] +
             recbase[(17 + a) * 32 + l] * recbase[(50 + h) * 32 + l];
    } else if (pidx < 288) {
      const int h = pidx - 272;
      for (int l = 0; l < 32; ++l) s += recbase[(34 + h) * 32 + l];
    } else if (pidx < 544) {
      const int a = (pidx - 288) >> 4, h = (pidx - 288) & 15;
      for (int l = 0; l < 32; ++l)
        s += recbase[(66 + a) * 32 + l] * recbase[(98 + h) * 32 + l] +
             recbase[(82 + a) * 32 + l] * recbase[(114 + h) * 32 + l];
    } else if (pidx < 560) {
      const int h = pidx - 544;
      for (int l = 0; l < 32; ++l) s += recbase[(98 + h) * 32 + l];
    } else if (pidx < 576) {
      const int h = pidx - 560;
      for (int l = 0; l < 32; ++l) s += recbase[(130 + h) * 32 + l];
    } else {
      for (int l = 0; l < 32; ++l) s += recbase[146 * 32 + l];
    }
    acc[q] += (double)s;
  }
}

// Copy the weights of a by-value MlpParams into shared memory (one warp or CTA).
__device__ inline void stage_mlp_weights(const MlpParams& m, float* dst, int tid, int nthreads) {
  const float* src = reinterpret_cast<const float*>(&m);
  for (int i = tid; i < kMlpFloats; i += nthreads) dst[i] = (i < 577) ? src[i] : 0.0f;
}

// Host: copy the flat HOST parameter vector of a qex_xc_spec into MlpParams.
inline bool fill_mlp_params(MlpParams& m, const qex_xc_spec* xc) {
  if (!xc || !xc->mlp_params_host || !(xc->normalization != 0.0)) return false;
  const float* q = xc->mlp_params_host;
  memcpy(m.w1, q, sizeof(m.w1));
  q += QEX_MLP_WINDOW * QEX_MLP_HIDDEN;
  memcpy(m.b1, q, sizeof(m.b1));
  q += QEX_MLP_HIDDEN;
  memcpy(m.w2, q, sizeof(m.w2));
  q += QEX_MLP_HIDDEN * QEX_MLP_HIDDEN;
  memcpy(m.b2, q, sizeof(m.b2));
  q += QEX_MLP_HIDDEN;
  memcpy(m.w3, q, sizeof(m.w3));
  q += QEX_MLP_HIDDEN;
  m.b3 = q[0];
  m.norm_inv = (float)(1.0 / xc->normalization);
  return true;
}

}  // namespace qex
