// Warp-level evaluation of the reference's dense XC networks inside the 1D
// kernels: LocalMLP and GlobalMLP of qedft/models/networks.py:83-138
// (stax Dense stacks of qedft/models/classical/classical_models.py:77-224),
// with the wrappers of qedft/models/wrappers.py:162-217 (jax_dft's
// self-interaction layer and negativity transform, then the mean over the
// grid for global networks).
//
// Network (FP32): x -> [Dense(H) -> act] x L -> Dense(1), x = n / norm.
//   local  (QEX_XC_LOCAL_MLP):  x = n_i, one scalar per grid point, g_i = MLP(n_i / norm);
//   global (QEX_XC_GLOBAL_MLP): x = n (all N points), one scalar g = MLP(n / norm).
// Wrappers (FP64): u_i = beta (-v_H[n]_i / 2) + (1 - beta) g_i with
//   beta = exp(-((dx sum n - 1) / width)^2)  (self-interaction, optional);
//   f_i = -swish(u_i)                        (negativity, optional);
//   global networks return mean_i f_i, stored here as per-point values f_i / N
//   so that the sum over the grid is the network's scalar (the amplitude
//   convention's E_xc = dx sum values).
// The potential is the exact derivative of E_xc: forward-mode (value and
// tangent) through the local network, reverse mode through the global one,
// and the Hartree term of the self-interaction layer by the symmetric kernel
// (sum_i c_i dv_H,i/dn_j = v_H[c]_j).
//
// Packed FP32 parameters (device, 16-byte aligned; H padded to Hp, a multiple
// of 8, with zero weights): W1 (inputs x Hp), b1 (Hp), then for each further
// hidden layer W (Hp x Hp), b (Hp), then Wout (Hp), then {bout, width, 0, 0}.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "ks1d_common.cuh"
#include "qex_ks1d.h"

namespace qex {

constexpr int kNnMaxWidth = 128;

struct NnNet {
  const float* P;
  int H;       // padded hidden width (multiple of 8, <= kNnMaxWidth)
  int L;       // hidden layers (>= 1)
  int act;     // enum qex_nn_activation
  int inputs;  // 1 (local) or the grid size (global)
  int flags;   // QEX_NN_SELF_INTERACTION | QEX_NN_NEGATIVITY
  float norm;  // density_normalization_factor: x = n / norm
  double si_amp, si_rho_per_dx;  // exponential interaction A exp(-k |d|): A and k
};

__host__ __device__ inline long long nn_off_b1(const NnNet& n) { return (long long)n.inputs * n.H; }
// W of hidden layer l (l >= 1; layer 0 is W1)
__host__ __device__ inline long long nn_off_w(const NnNet& n, int l) {
  return nn_off_b1(n) + n.H + (long long)(l - 1) * ((long long)n.H * n.H + n.H);
}
__host__ __device__ inline long long nn_off_b(const NnNet& n, int l) {
  return l == 0 ? nn_off_b1(n) : nn_off_w(n, l) + (long long)n.H * n.H;
}
__host__ __device__ inline long long nn_off_out(const NnNet& n) { return nn_off_w(n, n.L); }
__host__ __device__ inline long long nn_num_floats(const NnNet& n) { return nn_off_out(n) + n.H + 4; }

inline bool is_nn_kind(int kind) { return kind == QEX_XC_LOCAL_MLP || kind == QEX_XC_GLOBAL_MLP; }

// Validates the dense-network fields of a spec and fills the device view.
inline int fill_nn(NnNet& n, const qex_xc_spec* xc) {
  if (!xc->nn_params || reinterpret_cast<uintptr_t>(xc->nn_params) % 16 != 0) return QEX_BAD_ARG;
  if (xc->nn_width < 8 || xc->nn_width > QEX_NN_MAX_WIDTH || xc->nn_width % 8 != 0)
    return QEX_BAD_ARG;
  if (xc->nn_layers < 1 || xc->nn_layers > 64) return QEX_BAD_ARG;
  if (xc->nn_activation < QEX_NN_TANH || xc->nn_activation > QEX_NN_GELU) return QEX_BAD_ARG;
  if ((xc->nn_flags & ~(QEX_NN_SELF_INTERACTION | QEX_NN_NEGATIVITY)) != 0) return QEX_BAD_ARG;
  if (xc->kind == QEX_XC_LOCAL_MLP ? xc->nn_inputs != 1 : xc->nn_inputs < 1) return QEX_BAD_ARG;
  if (!(xc->normalization != 0.0) || !isfinite(xc->normalization)) return QEX_BAD_ARG;
  n.P = xc->nn_params;
  n.H = xc->nn_width;
  n.L = xc->nn_layers;
  n.act = xc->nn_activation;
  n.inputs = xc->nn_inputs;
  n.flags = xc->nn_flags;
  n.norm = (float)xc->normalization;
  // the self-interaction layer's Hartree term uses jax_dft's exponential
  // Coulomb interaction with its default constants (qedft/models/wrappers.py:188-192)
  n.si_amp = 1.071295;
  n.si_rho_per_dx = 1.0 / 2.385345;
  return QEX_OK;
}

// FP32 activation and its derivative (the stax layers of classical_models.py:37-47).
__device__ inline float nn_act(int act, float z, float& d) {
  switch (act) {
    case QEX_NN_RELU:
      d = z > 0.0f ? 1.0f : 0.0f;
      return fmaxf(z, 0.0f);
    case QEX_NN_SOFTPLUS: {  // log(1 + e^z), computed as max(z, 0) + log1p(e^-|z|)
      const float e = expf(-fabsf(z));
      d = z >= 0.0f ? 1.0f / (1.0f + e) : e / (1.0f + e);
      return fmaxf(z, 0.0f) + log1pf(e);
    }
    case QEX_NN_SIGMOID: {
      const float e = expf(-fabsf(z));
      const float s = z >= 0.0f ? 1.0f / (1.0f + e) : e / (1.0f + e);
      d = s * (1.0f - s);
      return s;
    }
    case QEX_NN_ELU:
      if (z > 0.0f) {
        d = 1.0f;
        return z;
      }
      d = expf(z);
      return expm1f(z);
    case QEX_NN_LEAKY_RELU:
      d = z >= 0.0f ? 1.0f : 0.01f;
      return z >= 0.0f ? z : 0.01f * z;
    case QEX_NN_SELU: {
      const float a = 1.6732632423543772f, s = 1.0507009873554805f;
      if (z > 0.0f) {
        d = s;
        return s * z;
      }
      d = s * a * expf(z);
      return s * a * expm1f(z);
    }
    case QEX_NN_GELU: {  // tanh approximation (jax.nn.gelu, approximate=True)
      const float c = 0.7978845608028654f, k = 0.044715f;
      const float t = tanhf(c * (z + k * z * z * z));
      d = 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * c * (1.0f + 3.0f * k * z * z);
      return 0.5f * z * (1.0f + t);
    }
    default: {  // tanh
      const float t = tanhf(z);
      d = 1.0f - t * t;
      return t;
    }
  }
}

// Local network at one point per lane: returns g = MLP(x) and, with kTan,
// gp = dg/dx.  buf: this lane's scratch (lane-interleaved, stride 32):
// 4 Hp floats (value and tangent of two layers, ping-pong).
template <bool kTan>
__device__ inline float nn_local_point(const NnNet& net, float x, float& gp, float* buf) {
  const int H = net.H;
  float* cur = buf;
  float* nxt = buf + 2 * H * kWarp;
  {
    const float* W = net.P;
    const float* B = net.P + nn_off_b1(net);
#pragma unroll 1
    for (int k = 0; k < H; ++k) {
      const float w = __ldg(W + k);
      float d;
      const float h = nn_act(net.act, fmaf(x, w, __ldg(B + k)), d);
      cur[k * kWarp] = h;
      if (kTan) cur[(H + k) * kWarp] = d * w;
    }
  }
#pragma unroll 1
  for (int l = 1; l < net.L; ++l) {
    const float* W = net.P + nn_off_w(net, l);
    const float* B = net.P + nn_off_b(net, l);
#pragma unroll 1
    for (int c = 0; c < H; c += 8) {
      float z[8], dz[8];
      const float4 b0 = __ldg(reinterpret_cast<const float4*>(B + c));
      const float4 b1 = __ldg(reinterpret_cast<const float4*>(B + c + 4));
      z[0] = b0.x; z[1] = b0.y; z[2] = b0.z; z[3] = b0.w;
      z[4] = b1.x; z[5] = b1.y; z[6] = b1.z; z[7] = b1.w;
#pragma unroll
      for (int e = 0; e < 8; ++e) dz[e] = 0.0f;
#pragma unroll 2
      for (int k = 0; k < H; ++k) {
        const float hk = cur[k * kWarp];
        const float4 w0 = __ldg(reinterpret_cast<const float4*>(W + (long long)k * H + c));
        const float4 w1 = __ldg(reinterpret_cast<const float4*>(W + (long long)k * H + c + 4));
        const float w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
        for (int e = 0; e < 8; ++e) z[e] = fmaf(hk, w[e], z[e]);
        if (kTan) {
          const float dk = cur[(H + k) * kWarp];
#pragma unroll
          for (int e = 0; e < 8; ++e) dz[e] = fmaf(dk, w[e], dz[e]);
        }
      }
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        float d;
        nxt[(c + e) * kWarp] = nn_act(net.act, z[e], d);
        if (kTan) nxt[(H + c + e) * kWarp] = d * dz[e];
      }
    }
    float* t = cur;
    cur = nxt;
    nxt = t;
  }
  const float* Wo = net.P + nn_off_out(net);
  float g = __ldg(Wo + H), dg = 0.0f;
#pragma unroll 1
  for (int k = 0; k < H; ++k) {
    const float w = __ldg(Wo + k);
    g = fmaf(cur[k * kWarp], w, g);
    if (kTan) dg = fmaf(cur[(H + k) * kWarp], w, dg);
  }
  gp = dg;
  return g;
}

// Global network forward over the warp.  x: the N inputs (FP32, shared,
// already divided by norm).  zs: L x Hp pre-activations (shared, out);
// h: Hp floats (shared scratch).  Returns g on every lane.
__device__ inline float nn_global_forward(const NnNet& net, const float* x, int N, float* zs,
                                          float* h, int lane) {
  const int H = net.H;
  for (int u0 = 0; u0 < H; u0 += kWarp) {
    const int u = u0 + lane;
    if (u < H) {
      const float* W = net.P;
      float a0 = __ldg(net.P + nn_off_b1(net) + u), a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
      int i = 0;
#pragma unroll 1
      for (; i + 4 <= N; i += 4) {
        a0 = fmaf(x[i], __ldg(W + (long long)i * H + u), a0);
        a1 = fmaf(x[i + 1], __ldg(W + (long long)(i + 1) * H + u), a1);
        a2 = fmaf(x[i + 2], __ldg(W + (long long)(i + 2) * H + u), a2);
        a3 = fmaf(x[i + 3], __ldg(W + (long long)(i + 3) * H + u), a3);
      }
      for (; i < N; ++i) a0 = fmaf(x[i], __ldg(W + (long long)i * H + u), a0);
      zs[u] = (a0 + a1) + (a2 + a3);
    }
  }
  __syncwarp();
#pragma unroll 1
  for (int l = 1; l < net.L; ++l) {
    for (int u = lane; u < H; u += kWarp) {
      float d;
      h[u] = nn_act(net.act, zs[(l - 1) * H + u], d);
    }
    __syncwarp();
    const float* W = net.P + nn_off_w(net, l);
    for (int u = lane; u < H; u += kWarp) {
      float a = __ldg(net.P + nn_off_b(net, l) + u);
#pragma unroll 4
      for (int k = 0; k < H; ++k) a = fmaf(h[k], __ldg(W + (long long)k * H + u), a);
      zs[l * H + u] = a;
    }
    __syncwarp();
  }
  const float* Wo = net.P + nn_off_out(net);
  float part = 0.0f;
  for (int u = lane; u < H; u += kWarp) {
    float d;
    part = fmaf(nn_act(net.act, zs[(net.L - 1) * H + u], d), __ldg(Wo + u), part);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(kFull, part, o);
  return part + __ldg(Wo + H);
}

// Global network backward: gx[i] = d g / d x_i for i < N (FP32, written to
// gx, any memory).  zs from nn_global_forward; dl, dn: Hp floats each (shared).
__device__ inline void nn_global_backward(const NnNet& net, const float* zs, int N, float* dl,
                                          float* dn, float* gx, int lane) {
  const int H = net.H;
  const float* Wo = net.P + nn_off_out(net);
  for (int u = lane; u < H; u += kWarp) {
    float d;
    nn_act(net.act, zs[(net.L - 1) * H + u], d);
    dl[u] = __ldg(Wo + u) * d;
  }
  __syncwarp();
#pragma unroll 1
  for (int l = net.L - 1; l >= 1; --l) {
    const float* W = net.P + nn_off_w(net, l);
    for (int k = lane; k < H; k += kWarp) {
      float a = 0.0f;
#pragma unroll 1
      for (int u = 0; u < H; u += 4) {
        const float4 w = __ldg(reinterpret_cast<const float4*>(W + (long long)k * H + u));
        a = fmaf(w.x, dl[u], a);
        a = fmaf(w.y, dl[u + 1], a);
        a = fmaf(w.z, dl[u + 2], a);
        a = fmaf(w.w, dl[u + 3], a);
      }
      float d;
      nn_act(net.act, zs[(l - 1) * H + k], d);
      dn[k] = a * d;
    }
    __syncwarp();
    for (int k = lane; k < H; k += kWarp) dl[k] = dn[k];
    __syncwarp();
  }
#pragma unroll 1
  for (int i = lane; i < N; i += kWarp) {
    float a = 0.0f;
    const float* row = net.P + (long long)i * H;
#pragma unroll 1
    for (int u = 0; u < H; u += 4) {
      const float4 w = __ldg(reinterpret_cast<const float4*>(row + u));
      a = fmaf(w.x, dl[u], a);
      a = fmaf(w.y, dl[u + 1], a);
      a = fmaf(w.z, dl[u + 2], a);
      a = fmaf(w.w, dl[u + 3], a);
    }
    gx[i] = a;
  }
  __syncwarp();
}

// out_i = dx sum_j n_j A r^|i-j|, r = exp(-k dx): the forward and backward
// recurrences F_i = n_i + r F_{i-1}, B_i = n_i + r B_{i+1} (out = A dx (F + B - n)),
// each lane running one contiguous chunk and the chunk carries joined by an
// exclusive warp scan of the affine maps.  n and out are distinct (out may be
// global memory; F is parked in out between the two sweeps).
__device__ inline void nn_exp_hartree(const double* n, int N, double dx, double A, double k,
                                      double* out, int lane) {
  const double r = exp(-k * dx);
  const int C = (N + kWarp - 1) / kWarp;
  const int beg = min(lane * C, N), end = min(beg + C, N);
  // forward
  double s = 0.0, f = 1.0;
#pragma unroll 1
  for (int i = beg; i < end; ++i) {
    s = fma(s, r, n[i]);
    f *= r;
  }
  // exclusive scan of (f, s): carry_in of lane = composition of lanes < lane
  double cs = s, cf = f;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    const double ps = __shfl_up_sync(kFull, cs, o), pf = __shfl_up_sync(kFull, cf, o);
    if (lane >= o) {
      cs = fma(ps, cf, cs);
      cf *= pf;
    }
  }
  double carry = __shfl_up_sync(kFull, cs, 1);
  if (lane == 0) carry = 0.0;
#pragma unroll 1
  for (int i = beg; i < end; ++i) {
    carry = fma(carry, r, n[i]);
    out[i] = carry;
  }
  // backward
  s = 0.0;
  f = 1.0;
#pragma unroll 1
  for (int i = end - 1; i >= beg; --i) {
    s = fma(s, r, n[i]);
    f *= r;
  }
  cs = s;
  cf = f;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    const double ps = __shfl_down_sync(kFull, cs, o), pf = __shfl_down_sync(kFull, cf, o);
    if (lane + o < kWarp) {
      cs = fma(ps, cf, cs);
      cf *= pf;
    }
  }
  carry = __shfl_down_sync(kFull, cs, 1);
  if (lane == kWarp - 1) carry = 0.0;
  const double ad = A * dx;
#pragma unroll 1
  for (int i = end - 1; i >= beg; --i) {
    carry = fma(carry, r, n[i]);
    out[i] = ad * (out[i] + carry - n[i]);
  }
  __syncwarp();
}

// FP32 shared floats nn_xc needs (beyond the density it is given).
__host__ __device__ inline long long nn_smem_floats(int kind, int H, int L, int nmax) {
  if (kind == QEX_XC_LOCAL_MLP) return 4LL * H * kWarp;
  return (long long)nmax + (long long)L * H + 3LL * H + 4;
}

// E_xc (dx included) of a dense network on the density n (N points, FP64,
// any memory), and with want_v its potential in vout (amplitude: dE/dn;
// local: (dE/dn)/dx).  frec (optional): the per-point values.  s32: the
// shared floats of nn_smem_floats.  g, gp, vs, c: four N-double scratch
// vectors (global).  Returns the same value on every lane.
__device__ inline double nn_xc_eval(const NnNet& net, int kind, int N, double dx, bool local_conv,
                                    const double* n, bool want_v, double* vout, double* frec,
                                    float* s32, double* g, double* gp, double* vs, double* c,
                                    int lane) {
  const bool si = (net.flags & QEX_NN_SELF_INTERACTION) != 0;
  const bool neg = (net.flags & QEX_NN_NEGATIVITY) != 0;
  const bool global = kind == QEX_XC_GLOBAL_MLP;
  // ---- network (FP32)
  double gscal = 0.0;
  if (!global) {
    float* buf = s32 + lane;
    for (int r0 = 0; r0 < N; r0 += kWarp) {
      const int i = r0 + lane;
      const float x = i < N ? (float)n[i] / net.norm : 0.0f;
      float d = 0.0f;
      const float y = want_v ? nn_local_point<true>(net, x, d, buf)
                             : nn_local_point<false>(net, x, d, buf);
      if (i < N) {
        g[i] = (double)y;
        gp[i] = (double)d / (double)net.norm;
      }
    }
  } else {
    float* x = s32;
    float* zs = x + N;
    float* h = zs + net.L * net.H;
    float* d2 = h + net.H;
    for (int i = lane; i < N; i += kWarp) x[i] = (float)n[i] / net.norm;
    __syncwarp();
    gscal = (double)nn_global_forward(net, x, N, zs, h, lane);
    if (want_v) {
      float* gx = x;  // the inputs are dead after the forward pass
      nn_global_backward(net, zs, N, h, d2, gx, lane);
      for (int i = lane; i < N; i += kWarp) gp[i] = (double)gx[i] / (double)net.norm;
    }
  }
  __syncwarp();
  // ---- wrappers and energy (FP64)
  double q = 0.0;
  for (int i = lane; i < N; i += kWarp) q += n[i];
  q = warp_sum(q) * dx;
  double beta = 0.0, width = 1.0;
  if (si) {
    width = (double)__ldg(net.P + nn_off_out(net) + net.H + 1);
    const double t = (q - 1.0) / width;
    beta = exp(-t * t);
    nn_exp_hartree(n, N, dx, net.si_amp, net.si_rho_per_dx, vs, lane);
  }
  const double wsc = global ? 1.0 / (double)N : 1.0;
  double e = 0.0, csum = 0.0, tsi = 0.0;
  for (int i = lane; i < N; i += kWarp) {
    const double gi = global ? gscal : g[i];
    const double u = si ? fma(-0.5 * beta, vs[i], (1.0 - beta) * gi) : gi;
    double f = u, fp = 1.0;
    if (neg) {
      const double s = 1.0 / (1.0 + exp(-u));
      f = -u * s;
      fp = -(s + u * s * (1.0 - s));
    }
    const double val = f * wsc;
    if (frec) frec[i] = val;
    const double w = local_conv ? n[i] : 1.0;
    e = fma(val, w, e);
    if (want_v) {
      const double ci = w * wsc * fp;
      c[i] = ci;
      csum += ci;
      if (si) tsi = fma(ci, -0.5 * vs[i] - gi, tsi);
      if (local_conv) vout[i] = val;  // the direct term of E = dx sum val n
    }
  }
  e = warp_sum(e) * dx;
  if (!want_v) return e;
  csum = warp_sum(csum);
  tsi = warp_sum(tsi);
  __syncwarp();
  const double dbeta = si ? beta * (-2.0 * (q - 1.0) / (width * width)) * dx : 0.0;
  if (si) nn_exp_hartree(c, N, dx, net.si_amp, net.si_rho_per_dx, g, lane);  // g <- v_H[c]
  const double keep = si ? 1.0 - beta : 1.0;
  for (int i = lane; i < N; i += kWarp) {
    double t = global ? keep * csum * gp[i] : keep * c[i] * gp[i];
    if (si) t += fma(-0.5 * beta, g[i], tsi * dbeta);
    // dE/dn_i = dx (direct + t); local convention v = (dE/dn)/dx
    const double direct = local_conv ? vout[i] : 0.0;
    vout[i] = local_conv ? direct + t : dx * t;
  }
  __syncwarp();
  return e;
}

}  // namespace qex
