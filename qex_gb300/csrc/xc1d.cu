// Point-parallel evaluation of the 1D exchange-correlation functionals on
// packed densities: per-point values f, the potential v_xc and E_xc per
// molecule.  One CTA per molecule; any grid size.
//
// Reference: qedft/train/od/scf.py:32-76 (get_xc_energy_amplitude_encoded /
// get_xc_potential_amplitude_encoded, the potential carries the factor dx) and
// the jax_dft local convention (E = dx sum f n, v = (dE/dn)/dx).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "ks1d_common.cuh"
#include "ksr_device.cuh"
#include "nn_device.cuh"
#include "qex_xc1d.h"
#include "xc_device.cuh"

namespace qex {
namespace {

struct XcParams {
  int num_molecules;
  const int32_t* num_grids;
  const int64_t* offsets;
  const double* spacing;
  const double* density;
  double* values;
  double* potential;
  double* energy;
  float* grad;  // (total points, 17) window gradients, MLP only
  int kind, conv;
  double a, p, shift, lda_A, lda_kappa;
  MlpParams mlp;
};

constexpr int kThreads = 64;

__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < kWarp) {
    t = (threadIdx.x < kThreads / kWarp) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
  }
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kThreads) xc1d_kernel(const __grid_constant__ XcParams p) {
  __shared__ double red[kThreads / kWarp];
  __shared__ __align__(16) float wsm[kMlpFloats];
  __shared__ float wbuf[QEX_MLP_WINDOW * kThreads];
  __shared__ float sbuf[kMlpScratch * kThreads];
  if (p.kind == QEX_XC_WINDOW_MLP) stage_mlp_weights(p.mlp, wsm, threadIdx.x, kThreads);
  __syncthreads();
  const int b = blockIdx.x;
  if (b >= p.num_molecules) return;
  const int N = p.num_grids[b];
  const long long off = p.offsets[b];
  const double dx = p.spacing[b];
  const double* n = p.density + off;
  const bool local = p.conv == QEX_XC_LOCAL;
  double e = 0.0;
  if (p.kind == QEX_XC_WINDOW_MLP) {
    const float ninv = p.mlp.norm_inv;
    for (int i = threadIdx.x; i < N; i += kThreads) {
#pragma unroll
      for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
        int j = i - kPadMlp + k;
        wbuf[k * kThreads + threadIdx.x] = (j >= 0 && j < N) ? (float)n[j] * ninv : 0.0f;
      }
      float* scr = sbuf + threadIdx.x;
      float f = mlp_point<true>(wsm, wbuf + threadIdx.x, kThreads, scr, kThreads);
      if (p.values) p.values[off + i] = (double)f;
      e += local ? (double)f * n[i] : (double)f;
      const float up = local ? (float)n[i] * ninv : ninv;
      for (int k = 0; k < QEX_MLP_WINDOW; ++k)
        p.grad[(off + i) * QEX_MLP_WINDOW + k] = up * scr[k * kThreads];
    }
    __syncthreads();
    if (p.potential) {
      for (int j = threadIdx.x; j < N; j += kThreads) {
        // v_j = sum over points i with window offset k = j - i + 8
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
          int i = j + kPadMlp - k;
          if (i >= 0 && i < N) acc += p.grad[(off + i) * QEX_MLP_WINDOW + k];
        }
        double v = (double)acc;
        if (local) v += p.values ? p.values[off + j] : 0.0;
        p.potential[off + j] = local ? v : dx * v;
      }
    }
  } else {
    for (int i = threadIdx.x; i < N; i += kThreads) {
      double ni = n[i], f = 0.0, df = 0.0;
      if (p.kind == QEX_XC_LDA_EXP_COULOMB) {
        lda_exp_coulomb<true>(ni, lda_consts(p.lda_A, p.lda_kappa), f, df);
      } else if (p.kind == QEX_XC_POWER) {
        double base = ni + p.shift;
        f = p.a * pow(base, p.p);
        df = p.a * p.p * pow(base, p.p - 1.0);
      }
      if (p.values) p.values[off + i] = f;
      if (local) {
        e = fma(f, ni, e);
        if (p.potential) p.potential[off + i] = fma(ni, df, f);
      } else {
        e += f;
        if (p.potential) p.potential[off + i] = dx * df;
      }
    }
  }
  e = block_sum(e, red);
  if (threadIdx.x == 0 && p.energy) p.energy[b] = e * dx;
}

struct KsrEvalParams {
  int num_molecules;
  const int32_t* num_grids;
  const int64_t* offsets;
  const double* spacing;
  const double* density;
  double* values;
  double* potential;
  double* energy;
  int conv;
  int nmax;
  int channels;
  int slot;
  const float* w;
  double lo, hi;
};

template <int C>
__device__ double ksr_one(const KsrEvalParams& p, int N, double dx, long long off, bool local,
                          double* vals, float* scratch, int lane) {
  return p.potential ? ksr_eval<C, true, 4>(p.w, p.slot, p.lo, p.hi, N, dx, p.density + off, local,
                                         p.potential + off, vals, scratch, lane)
                     : ksr_eval<C, false, 4>(p.w, p.slot, p.lo, p.hi, N, dx, p.density + off, local,
                                          nullptr, vals, scratch, lane);
}

// One warp per molecule; the warp-level evaluation shared with the SCF kernel.
__global__ void __launch_bounds__(kWarp) ksr1d_kernel(const __grid_constant__ KsrEvalParams p) {
  extern __shared__ __align__(16) float ksm[];
  const int b = blockIdx.x;
  const int lane = threadIdx.x;
  if (b >= p.num_molecules) return;
  const int N = p.num_grids[b];
  if (N < 1 || N > p.nmax) {
    if (lane == 0 && p.energy) p.energy[b] = nan("");
    return;
  }
  const long long off = p.offsets[b];
  const double dx = p.spacing[b];
  const bool local = p.conv == QEX_XC_LOCAL;
  double* vals = p.values ? p.values + off : nullptr;
  double e = p.channels == 16 ? ksr_one<16>(p, N, dx, off, local, vals, ksm, lane)
                              : ksr_one<8>(p, N, dx, off, local, vals, ksm, lane);
  e = warp_sum(e);
  if (lane == 0 && p.energy) p.energy[b] = e * dx;
}

struct NnEvalParams {
  int num_molecules;
  const int32_t* num_grids;
  const int64_t* offsets;
  const double* spacing;
  const double* density;
  double* values;
  double* potential;
  double* energy;
  int kind, conv;
  NnNet net;
  double* scratch;  // 4 vectors per molecule: molecule b at 4 * offsets[b]
};

// Dense networks (LocalMLP / GlobalMLP): one warp per molecule, the
// warp-level evaluation shared with the SCF kernel.
__global__ void __launch_bounds__(kWarp) nn1d_kernel(const __grid_constant__ NnEvalParams p) {
  extern __shared__ __align__(16) float nsm[];
  const int b = blockIdx.x;
  const int lane = threadIdx.x;
  if (b >= p.num_molecules) return;
  const int N = p.num_grids[b];
  if (N < 1 || (p.kind == QEX_XC_GLOBAL_MLP && N != p.net.inputs)) {
    if (lane == 0 && p.energy) p.energy[b] = nan("");
    return;
  }
  const long long off = p.offsets[b];
  const double dx = p.spacing[b];
  double* sc = p.scratch + 4 * off;
  const double e = nn_xc_eval(p.net, p.kind, N, dx, p.conv == QEX_XC_LOCAL, p.density + off,
                              p.potential != nullptr, p.potential ? p.potential + off : nullptr,
                              p.values ? p.values + off : nullptr, nsm, sc, sc + N, sc + 2 * N,
                              sc + 3 * N, lane);
  if (lane == 0 && p.energy) p.energy[b] = e;
}

}  // namespace
}  // namespace qex

extern "C" {

int qex_ksr1d_eval(int32_t num_molecules, int32_t max_num_grids, const int32_t* num_grids,
                   const int64_t* grid_offsets, const double* grid_spacing,
                   const qex_xc_spec* xc, const double* density, double* values,
                   double* potential, double* energy, void* stream) {
  using namespace qex;
  if (num_molecules < 0 || !xc || xc->kind != QEX_XC_KSR) return QEX_BAD_ARG;
  if (xc->convention != QEX_XC_AMPLITUDE && xc->convention != QEX_XC_LOCAL) return QEX_BAD_ARG;
  if (num_molecules == 0) return QEX_OK;
  if (!num_grids || !grid_offsets || !grid_spacing || !density || max_num_grids < 1)
    return QEX_BAD_ARG;
  if (!xc->ksr_params || reinterpret_cast<uintptr_t>(xc->ksr_params) % 16 != 0) return QEX_BAD_ARG;
  if (!(xc->ksr_maxval >= xc->ksr_minval) || !(xc->ksr_minval > 0.0)) return QEX_BAD_ARG;
  if (xc->ksr_channels != 8 && xc->ksr_channels != 16) return QEX_BAD_ARG;
  const size_t smem = sizeof(float) * ksr_scratch_floats(max_num_grids);
  int dev = 0, max_optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)max_optin) return QEX_BAD_ARG;
  if (cudaFuncSetAttribute(ksr1d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return QEX_CUDA_ERROR;
  KsrEvalParams P;
  memset(&P, 0, sizeof(P));
  P.num_molecules = num_molecules;
  P.num_grids = num_grids;
  P.offsets = grid_offsets;
  P.spacing = grid_spacing;
  P.density = density;
  P.values = values;
  P.potential = potential;
  P.energy = energy;
  P.conv = xc->convention;
  P.nmax = max_num_grids;
  P.channels = xc->ksr_channels;
  P.w = xc->ksr_params;
  P.lo = xc->ksr_minval;
  P.hi = xc->ksr_maxval;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto stage =
      ksr_stage(xc->ksr_params, 6 * xc->ksr_channels * xc->ksr_channels + 2 * xc->ksr_channels, s);
  if (stage.capturing_refused()) return QEX_BAD_ARG;
  if (stage.slot() < 0) return QEX_CUDA_ERROR;
  P.slot = stage.slot();
  ksr1d_kernel<<<num_molecules, kWarp, smem, s>>>(P);
  if (cudaGetLastError() != cudaSuccess || !stage.finish()) return QEX_CUDA_ERROR;
  return QEX_OK;
}

int qex_xc1d_workspace_size(int64_t total_points, const qex_xc_spec* xc, size_t* bytes) {
  if (!bytes || !xc || total_points < 0) return QEX_BAD_ARG;
  *bytes = (xc->kind == QEX_XC_WINDOW_MLP)
               ? sizeof(float) * QEX_MLP_WINDOW * (size_t)total_points
               : 0;
  if (qex::is_nn_kind(xc->kind)) *bytes = sizeof(double) * 4 * (size_t)total_points;
  return QEX_OK;
}

int qex_xc1d_eval(int32_t num_molecules, int64_t total_points, const int32_t* num_grids,
                  const int64_t* grid_offsets, const double* grid_spacing,
                  const qex_xc_spec* xc, const double* density,
                  double* values, double* potential, double* energy, void* workspace,
                  size_t workspace_bytes, void* stream) {
  using namespace qex;
  if (num_molecules < 0 || !xc) return QEX_BAD_ARG;
  if (num_molecules == 0) return QEX_OK;
  if (!num_grids || !grid_offsets || !grid_spacing || !density) return QEX_BAD_ARG;
  if (is_nn_kind(xc->kind)) {
    if (xc->convention != QEX_XC_AMPLITUDE && xc->convention != QEX_XC_LOCAL) return QEX_BAD_ARG;
    NnEvalParams Q;
    memset(&Q, 0, sizeof(Q));
    if (fill_nn(Q.net, xc) != QEX_OK) return QEX_BAD_ARG;
    size_t need = 0;
    qex_xc1d_workspace_size(total_points, xc, &need);
    if (!workspace || workspace_bytes < need) return QEX_BAD_ARG;
    Q.num_molecules = num_molecules;
    Q.num_grids = num_grids;
    Q.offsets = grid_offsets;
    Q.spacing = grid_spacing;
    Q.density = density;
    Q.values = values;
    Q.potential = potential;
    Q.energy = energy;
    Q.kind = xc->kind;
    Q.conv = xc->convention;
    Q.scratch = static_cast<double*>(workspace);
    // the global network's input size is the grid size of every molecule
    const size_t smem =
        sizeof(float) * (size_t)nn_smem_floats(xc->kind, xc->nn_width, xc->nn_layers, xc->nn_inputs);
    int dev = 0, max_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem > (size_t)max_optin) return QEX_BAD_ARG;
    if (cudaFuncSetAttribute(nn1d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return QEX_CUDA_ERROR;
    nn1d_kernel<<<num_molecules, kWarp, smem, static_cast<cudaStream_t>(stream)>>>(Q);
    return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
  }
  if (xc->kind < QEX_XC_NONE || xc->kind > QEX_XC_WINDOW_MLP) return QEX_BAD_ARG;
  XcParams P;
  memset(&P, 0, sizeof(P));
  P.num_molecules = num_molecules;
  P.num_grids = num_grids;
  P.offsets = grid_offsets;
  P.spacing = grid_spacing;
  P.density = density;
  P.values = values;
  P.potential = potential;
  P.energy = energy;
  P.kind = xc->kind;
  P.conv = xc->convention;
  P.a = xc->coefficient;
  P.p = xc->power;
  P.shift = xc->shift;
  P.lda_A = xc->lda_amplitude;
  P.lda_kappa = xc->lda_kappa;
  if (xc->kind == QEX_XC_WINDOW_MLP) {
    if (!fill_mlp_params(P.mlp, xc)) return QEX_BAD_ARG;
    size_t need = 0;
    qex_xc1d_workspace_size(total_points, xc, &need);
    if (!workspace || workspace_bytes < need) return QEX_BAD_ARG;
    P.grad = static_cast<float*>(workspace);
    // the potential pass needs f in `values` for the local convention
    if (P.conv == QEX_XC_LOCAL && potential && !values) return QEX_BAD_ARG;
  }
  xc1d_kernel<<<num_molecules, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(P);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
