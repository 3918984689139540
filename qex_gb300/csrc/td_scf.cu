// Per-cycle bookkeeping of the 3D SCF as device kernels, so that a whole SCF
// runs without host synchronisation (and can be captured as one CUDA graph):
//   qex_td_fock_energy     F = h + J + V and E = tr(D h^T) + 1/2 tr(D J) + E_xc + E_nuc
//                          (hf.py:360-404 get_fock without DIIS; energy_tot,
//                          rks.py:149-163 / scf_functions_masked.py:243-265);
//   qex_td_orbital_gradient |g| with g = 2 C_vir^T F C_occ (pyscf rhf get_grad, as
//                          called at qedft/train/td/hf.py:81-84);
//   qex_td_scf_check       the reference's stop rule |E - E_last| < conv_tol and
//                          |g| < conv_tol_grad (hf.py:93-96), latching the
//                          cycle's results until the first converged cycle;
//   qex_td_aufbau_occ      get_occ (hf.py:602-607): 2 electrons in each of the
//                          lowest Ne/2 orbitals (ties by index);
//   qex_td_mask_pad / qex_td_mask_sort
//                          the padding and slot ordering of masked_generalized_eigh
//                          (generalized_eigensolver_masked.py:19-89).
// Every reduction is a fixed-order block reduction (deterministic).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kThreads = 1024;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <int kT>
__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < kT / 32) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kThreads) fock_energy_kernel(
    int n, const double* __restrict__ h, const double* __restrict__ J,
    const double* __restrict__ V, const double* __restrict__ D, const double* __restrict__ exc,
    double enuc, double* __restrict__ F, double* __restrict__ energy) {
  __shared__ double red[32];
  const long long nn = (long long)n * n;
  double s1 = 0.0, s2 = 0.0;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const double he = h[e], je = J[e];
    if (F) F[e] = he + je + V[e];
    const double d = D[e];
    s1 = fma(d, h[(long long)j * n + i], s1);
    s2 = fma(d, je, s2);
  }
  s1 = block_sum<kThreads>(s1, red);
  s2 = block_sum<kThreads>(s2, red);
  if (threadIdx.x == 0 && energy) energy[0] = s1 + 0.5 * s2 + (exc ? exc[0] : 0.0) + enuc;
}

// Y = F C_occ (columns of occupied orbitals; the others 0).
__global__ void fc_occ_kernel(int n, const double* __restrict__ F, const double* __restrict__ C,
                              const double* __restrict__ occ, double* __restrict__ Y) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e / n), j = (int)(e % n);
    double s = 0.0;
    if (occ[j] > 0.0) {
      const double* fr = F + (long long)k * n;
      for (int l = 0; l < n; ++l) s = fma(fr[l], C[(long long)l * n + j], s);
    }
    Y[e] = s;
  }
}

// partial[blk] = sum over (vir i, occ j) of this block's G_ij^2, G = C^T Y.
__global__ void __launch_bounds__(256) grad_part_kernel(int n, const double* __restrict__ C,
                                                        const double* __restrict__ occ,
                                                        const double* __restrict__ Y,
                                                        double* __restrict__ partial) {
  __shared__ double red[32];
  const long long nn = (long long)n * n;
  double acc = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (occ[i] > 0.0 || !(occ[j] > 0.0)) continue;
    double g = 0.0;
    for (int k = 0; k < n; ++k) g = fma(C[(long long)k * n + i], Y[(long long)k * n + j], g);
    g *= 2.0;
    acc = fma(g, g, acc);
  }
  acc = block_sum<256>(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(256) grad_sum_kernel(int parts, const double* __restrict__ partial,
                                                       double* __restrict__ norm) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < parts; i += blockDim.x) s += partial[i];
  s = block_sum<256>(s, red);
  if (threadIdx.x == 0) norm[0] = sqrt(s);
}

// state: [0] converged (0/1), [1] first converged cycle (-1), [2] cycles latched
__global__ void __launch_bounds__(kThreads) scf_check_kernel(
    int cycle, int n, const double* __restrict__ energies, const double* __restrict__ e_init,
    const double* __restrict__ gnorm, double conv_tol, double conv_tol_grad,
    int32_t* __restrict__ state, const double* __restrict__ dm, const double* __restrict__ mo_e,
    const double* __restrict__ mo_c, const double* __restrict__ occ, double* __restrict__ dm_out,
    double* __restrict__ mo_e_out, double* __restrict__ mo_c_out, double* __restrict__ occ_out,
    double* __restrict__ e_out) {
  __shared__ int latch;
  if (threadIdx.x == 0) {
    const bool before = state[0] != 0;
    latch = before ? 0 : 1;
    if (!before) {
      const double e = energies[cycle];
      const double el = cycle == 0 ? e_init[0] : energies[cycle - 1];
      if (fabs(e - el) < conv_tol && gnorm[0] < conv_tol_grad) {
        state[0] = 1;
        state[1] = cycle;
      }
      state[2] = cycle + 1;
      e_out[0] = e;
    }
  }
  __syncthreads();
  if (!latch) return;
  const long long nn = (long long)n * n;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    dm_out[e] = dm[e];
    mo_c_out[e] = mo_c[e];
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    mo_e_out[i] = mo_e[i];
    occ_out[i] = occ[i];
  }
}

__global__ void aufbau_kernel(int batch, int n, const double* __restrict__ e, int nocc,
                              double* __restrict__ occ) {
  const long long total = (long long)batch * n;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / n;
    const int i = (int)(t % n);
    const double* eb = e + b * n;
    const double ei = eb[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double ej = eb[j];
      rank += (ej < ei) || (ej == ei && j < i);
    }
    occ[t] = rank < nocc ? 2.0 : 0.0;
  }
}

// f = fock on the masked block, 1e-12 on padded diagonals, 0 elsewhere;
// s the same with s1e (generalized_eigensolver_masked.py:45-60)
__global__ void mask_pad_kernel(int n, const double* __restrict__ fock,
                                const double* __restrict__ s1e, const uint8_t* __restrict__ mask,
                                double* __restrict__ f, double* __restrict__ s) {
  const long long nn = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const bool mi = mask[i] != 0, mj = mask[j] != 0;
    const double pad = (!mi && i == j) ? 1e-12 : 0.0;
    f[e] = (mi && mj) ? fock[e] : pad;
    s[e] = (mi && mj) ? s1e[e] : pad;
  }
}

// Stable ascending order of key = (mask ? w : 1e12); w_out[rank] = w * mask,
// V_out[:, rank] = V[:, i] on the masked rows (0 on padded rows and columns).
__global__ void mask_sort_kernel(int n, const double* __restrict__ w, const double* __restrict__ V,
                                 const uint8_t* __restrict__ mask, double* __restrict__ w_out,
                                 double* __restrict__ V_out) {
  extern __shared__ int rank[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double ki = mask[i] ? w[i] : 1e12;
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double kj = mask[j] ? w[j] : 1e12;
      r += (kj < ki) || (kj == ki && j < i);
    }
    rank[i] = r;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) w_out[rank[i]] = mask[i] ? w[i] : 0.0;
  const long long nn = (long long)n * n;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int r = (int)(e / n), i = (int)(e % n);  // row r, source column i
    V_out[(long long)r * n + rank[i]] = (mask[r] && mask[i]) ? V[e] : 0.0;
  }
}

int grid_for(long long work, int threads) {
  long long g = (work + threads - 1) / threads;
  if (g > 4096) g = 4096;
  return (int)(g < 1 ? 1 : g);
}

constexpr int kGradParts = 512;

}  // namespace

extern "C" {

int qex_td_fock_energy(int32_t n, const double* h1e, const double* J, const double* V,
                       const double* dm, const double* excsum, double energy_nuc, double* fock,
                       double* energy, void* stream) {
  if (n < 1 || !h1e || !J || !V || !dm) return QEX_BAD_ARG;
  fock_energy_kernel<<<1, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      n, h1e, J, V, dm, excsum, energy_nuc, fock, energy);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

size_t qex_td_orbital_gradient_workspace_size(int32_t n) {
  return sizeof(double) * ((size_t)n * n + kGradParts);
}

int qex_td_orbital_gradient(int32_t n, const double* mo_coeff, const double* mo_occ,
                            const double* fock, double* norm, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (n < 1 || !mo_coeff || !mo_occ || !fock || !norm || !workspace) return QEX_BAD_ARG;
  if (workspace_bytes < qex_td_orbital_gradient_workspace_size(n)) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* Y = static_cast<double*>(workspace);
  double* part = Y + (size_t)n * n;
  const long long nn = (long long)n * n;
  fc_occ_kernel<<<grid_for(nn, 256), 256, 0, s>>>(n, fock, mo_coeff, mo_occ, Y);
  const int parts = grid_for(nn, 256) < kGradParts ? grid_for(nn, 256) : kGradParts;
  grad_part_kernel<<<parts, 256, 0, s>>>(n, mo_coeff, mo_occ, Y, part);
  grad_sum_kernel<<<1, 256, 0, s>>>(parts, part, norm);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_scf_check(int32_t cycle, int32_t n, const double* energies, const double* energy_init,
                     const double* gnorm, double conv_tol, double conv_tol_grad, int32_t* state,
                     const double* dm, const double* mo_energy, const double* mo_coeff,
                     const double* mo_occ, double* dm_out, double* mo_energy_out,
                     double* mo_coeff_out, double* mo_occ_out, double* energy_out, void* stream) {
  if (cycle < 0 || n < 1 || !energies || !energy_init || !gnorm || !state || !dm || !mo_energy ||
      !mo_coeff || !mo_occ || !dm_out || !mo_energy_out || !mo_coeff_out || !mo_occ_out ||
      !energy_out)
    return QEX_BAD_ARG;
  scf_check_kernel<<<1, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      cycle, n, energies, energy_init, gnorm, conv_tol, conv_tol_grad, state, dm, mo_energy,
      mo_coeff, mo_occ, dm_out, mo_energy_out, mo_coeff_out, mo_occ_out, energy_out);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_aufbau_occ(int32_t batch, int32_t n, const double* mo_energy, int32_t nelectron,
                      double* mo_occ, void* stream) {
  if (batch < 0 || n < 1 || nelectron < 0 || !mo_energy || !mo_occ) return QEX_BAD_ARG;
  if (batch == 0) return QEX_OK;
  aufbau_kernel<<<grid_for((long long)batch * n, 256), 256, 0,
                  static_cast<cudaStream_t>(stream)>>>(batch, n, mo_energy, nelectron / 2, mo_occ);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_mask_pad(int32_t n, const double* fock, const double* s1e, const uint8_t* mask,
                    double* fock_out, double* s1e_out, void* stream) {
  if (n < 1 || !fock || !s1e || !mask || !fock_out || !s1e_out) return QEX_BAD_ARG;
  mask_pad_kernel<<<grid_for((long long)n * n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, fock, s1e, mask, fock_out, s1e_out);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_mask_sort(int32_t n, const double* w, const double* V, const uint8_t* mask,
                     double* w_out, double* V_out, void* stream) {
  if (n < 1 || n > 8192 || !w || !V || !mask || !w_out || !V_out) return QEX_BAD_ARG;
  mask_sort_kernel<<<1, 1024, sizeof(int) * (size_t)n, static_cast<cudaStream_t>(stream)>>>(
      n, w, V, mask, w_out, V_out);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
