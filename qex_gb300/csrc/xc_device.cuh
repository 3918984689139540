// Device-side exchange-correlation building blocks shared by the 1D kernels.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "qex_ks1d.h"

namespace qex {

// Window-MLP weights, passed by value in kernel parameters so that every
// weight is a constant-bank operand of the FMA that uses it.
struct MlpParams {
  float w1[QEX_MLP_WINDOW * QEX_MLP_HIDDEN];
  float b1[QEX_MLP_HIDDEN];
  float w2[QEX_MLP_HIDDEN * QEX_MLP_HIDDEN];
  float b2[QEX_MLP_HIDDEN];
  float w3[QEX_MLP_HIDDEN];
  float b3;
  float norm_inv;
};

__device__ inline void lda_exp_coulomb(double n, double A, double kappa, double& eps,
                                       double& deps_dn) {
  // Exponential-Coulomb uniform-gas LDA (jax_dft xc.py, called at
  // qedft/train/od/eval.py:79; published fit of Baker et al., PRB 91, 235141).
  const double pi = 3.141592653589793;
  const double y = pi * n / kappa;
  const double ax = A / (2.0 * pi);
  double ex, dex;
  if (y > 1e-15) {
    double l = log1p(y * y);
    ex = ax * (l / y - 2.0 * atan(y));
    dex = -ax * l / (y * y);
  } else {
    ex = ax * (-y + y * y * y / 6.0);
    dex = ax * (-1.0 + 0.5 * y * y);
  }
  double ec, dec;
  if (y > 0.0) {
    const double sy = sqrt(y);
    const double c3 = pi * kappa * kappa / A;
    const double P = 2.0 - 1.00077 * sy + 6.26099 * y - 11.9041 * y * sy + 9.62614 * y * y -
                     1.48334 * y * y * sy + c3 * y * y * y;
    const double dP = -0.5 * 1.00077 / sy + 6.26099 - 1.5 * 11.9041 * sy + 2.0 * 9.62614 * y -
                      2.5 * 1.48334 * y * sy + 3.0 * c3 * y * y;
    ec = -A * y / pi / P;
    dec = -A / pi * (P - y * dP) / (P * P);
  } else {
    ec = 0.0;
    dec = -A / pi / 2.0;
  }
  eps = ex + ec;
  deps_dn = (dex + dec) * (pi / kappa);
}

__device__ inline float silu_d(float z, float& d) {
  float s = 1.0f / (1.0f + __expf(-z));
  d = s * (1.0f + z * (1.0f - s));
  return z * s;
}

// Window-MLP forward (and optionally input gradient) for one point.
// w: 17 inputs already divided by the normalization.
template <bool kGrad>
__device__ inline float mlp_point(const MlpParams& m, const float* w, float* gw) {
  float z1[QEX_MLP_HIDDEN], d1[QEX_MLP_HIDDEN], h1[QEX_MLP_HIDDEN];
#pragma unroll
  for (int h = 0; h < QEX_MLP_HIDDEN; ++h) {
    float z = m.b1[h];
#pragma unroll
    for (int k = 0; k < QEX_MLP_WINDOW; ++k) z = fmaf(w[k], m.w1[k * QEX_MLP_HIDDEN + h], z);
    z1[h] = z;
    h1[h] = silu_d(z, d1[h]);
  }
  float d2[QEX_MLP_HIDDEN];
  float out = m.b3;
#pragma unroll
  for (int h = 0; h < QEX_MLP_HIDDEN; ++h) {
    float z = m.b2[h];
#pragma unroll
    for (int k = 0; k < QEX_MLP_HIDDEN; ++k) z = fmaf(h1[k], m.w2[k * QEX_MLP_HIDDEN + h], z);
    float a = silu_d(z, d2[h]);
    out = fmaf(a, m.w3[h], out);
  }
  if (kGrad) {
    float g2[QEX_MLP_HIDDEN];
#pragma unroll
    for (int h = 0; h < QEX_MLP_HIDDEN; ++h) g2[h] = m.w3[h] * d2[h];
    float g1[QEX_MLP_HIDDEN];
#pragma unroll
    for (int k = 0; k < QEX_MLP_HIDDEN; ++k) {
      float a = 0.0f;
#pragma unroll
      for (int h = 0; h < QEX_MLP_HIDDEN; ++h) a = fmaf(m.w2[k * QEX_MLP_HIDDEN + h], g2[h], a);
      g1[k] = a * d1[k];
    }
#pragma unroll
    for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
      float a = 0.0f;
#pragma unroll
      for (int h = 0; h < QEX_MLP_HIDDEN; ++h) a = fmaf(m.w1[k * QEX_MLP_HIDDEN + h], g1[h], a);
      gw[k] = a;
    }
  }
  return out;
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
