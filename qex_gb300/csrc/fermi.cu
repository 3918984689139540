// Fractional (Fermi-Dirac) orbital occupations, qedft/train/td/fermi.py.
//
// One CTA per molecule, threads over orbitals.  The chemical potential mu is
// found by damped Newton steps on L(mu) = (N - F(mu))^2, F(mu) = sum_i 2 s_i,
// s_i = 1 / (1 + exp((e_i - mu) / theta)); each step needs F and its first two
// mu-derivatives, F' = sum 2 s(1-s) / theta and F'' = sum 2 s(1-s)(1-2s) / theta^2,
// reduced over the block in FP64 in a fixed order.  Modes follow the three
// reference implementations:
//   0  optimize_fermi_occupations (fermi.py:145-219): start e_0 + mu_shift,
//      stop once the loss < 1e-9, status QEX_NOT_CONVERGED if it ends > 1e-2;
//   1  get_fractional_occupations_jax (fermi.py:301-390): min(max_steps, 100)
//      steps, no early stop (a step that leaves mu unchanged ends the loop:
//      every later step would repeat it);
//   2  get_fractional_occupations_jax_stable (fermi.py:393-497): start at the
//      HOMO/LUMO midpoint; if the count misses by 1e-2 or more, ten
//      fixed-point steps at theta = 0.01 from the midpoint.
// Outputs per molecule: occupations (n), mu, the entropic energy
// theta sum 2 [f ln f + (1-f) ln(1-f)] (0 ln 0 taken as 0), the final loss.
#include <cuda_runtime.h>
#include <math.h>
#include <math_constants.h>
#include <stdint.h>

#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;

struct Sums {
  double f, f1, f2;
};

__device__ Sums block_sums(double a, double b, double c, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) {
    red[3 * w] = a;
    red[3 * w + 1] = b;
    red[3 * w + 2] = c;
  }
  __syncthreads();
  Sums s{0.0, 0.0, 0.0};
  for (int k = 0; k < kWarps; ++k) {  // every thread, same order
    s.f += red[3 * k];
    s.f1 += red[3 * k + 1];
    s.f2 += red[3 * k + 2];
  }
  __syncthreads();
  return s;
}

// F, F', F'' at mu (all threads get the block totals)
__device__ Sums fermi_sums(const double* e, int n, double mu, double theta, double* red) {
  double a = 0.0, b = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const double s = 1.0 / (1.0 + exp((e[i] - mu) / theta));
    const double q = s * (1.0 - s);
    a += 2.0 * s;
    b += 2.0 * q;
    c += 2.0 * q * (1.0 - 2.0 * s);
  }
  Sums t = block_sums(a, b, c, red);
  t.f1 /= theta;
  t.f2 /= theta * theta;
  return t;
}

__device__ double xlogx(double f) { return f > 0.0 ? f * log(f) : 0.0; }

struct FermiParams {
  int batch, n;
  const double* e;
  const double* nelec;
  double theta;
  const double* mu_in;  // NULL: the mode's default start
  double mu_shift, step;
  int max_steps, mode;
  double* occ;
  double* mu_out;
  double* entr;
  double* loss;
  int32_t* status;
};

__global__ void __launch_bounds__(kThreads) fermi_kernel(const __grid_constant__ FermiParams p) {
  __shared__ double red[3 * kWarps];
  const int b = blockIdx.x;
  if (b >= p.batch) return;
  const int n = p.n;
  const double* e = p.e + (long long)b * n;
  const double N = p.nelec[b];
  double theta = p.theta;

  // An electron count that is negative or not finite has no occupations: the
  // molecule's status says so and its outputs are NaN (the block takes this
  // branch as a whole, since N is one value per block).
  if (!(N >= 0.0) || !isfinite(N)) {
    for (int i = threadIdx.x; i < n; i += kThreads) p.occ[(long long)b * n + i] = CUDART_NAN;
    if (threadIdx.x == 0) {
      if (p.mu_out) p.mu_out[b] = CUDART_NAN;
      if (p.entr) p.entr[b] = CUDART_NAN;
      if (p.loss) p.loss[b] = CUDART_NAN;
      if (p.status) p.status[b] = QEX_BAD_ARG;
    }
    return;
  }
  // start.  HOMO and LUMO indices are clamped into [0, n) as the reference's
  // array lookup clamps them (fermi.py:422-427): more than 2n electrons take
  // the highest orbital for both.
  const double nd = floor(N / 2.0);
  const double rem = N - 2.0 * nd;
  const int n_double = (int)fmin(nd, (double)n);
  const int homo = min(max(n_double - 1, 0), n - 1);
  const int lumo = max(min(n_double + (rem > 0.0 ? 1 : 0), n - 1), 0);
  const double mid = 0.5 * (e[homo] + e[lumo]);
  double mu;
  if (p.mu_in) {
    mu = p.mu_in[b];
  } else {
    mu = (p.mode == 2) ? mid : e[0] + p.mu_shift;
  }
  const int steps = (p.mode == 0) ? p.max_steps : min(p.max_steps, 100);
  double loss = (p.mode == 0) ? 100.0 : 1.0;
  int st = QEX_OK;
  // iteration i evaluates at mu_i (after i updates): loss(mu_i), then updates
  for (int i = 0;; ++i) {
    const Sums t = fermi_sums(e, n, mu, theta, red);
    const double r = N - t.f;
    if (i > 0) loss = r * r;
    if (p.mode == 0 && i > 0 && loss < 1e-9) break;
    if (i >= steps) break;
    const double g = -2.0 * r * t.f1;
    const double gg = 2.0 * t.f1 * t.f1 - 2.0 * r * t.f2;
    double safe;
    if (p.mode == 0) {
      safe = fabs(gg) < 1e-10 ? 1e-10 * (double)((gg > 0.0) - (gg < 0.0)) : gg;
    } else if (p.mode == 1) {
      safe = (double)((gg > 0.0) - (gg < 0.0)) * fmax(fabs(gg), 1e-10);
    } else {
      safe = fabs(gg) < 1e-10 ? 1e-10 : gg;
    }
    const double next = mu - p.step * g / safe;
    if (p.mode != 0 && next == mu) {  // fixed point: the remaining steps repeat it
      loss = r * r;
      break;
    }
    mu = next;
  }
  if (p.mode == 0 && loss > 1e-2) st = QEX_NOT_CONVERGED;
  if (p.mode == 2) {
    loss = 0.0;
    const Sums t = fermi_sums(e, n, mu, theta, red);
    if (!(fabs(t.f - N) < 1e-2)) {
      theta = 0.01;
      mu = mid;
      for (int k = 0; k < 10; ++k) {
        const Sums u = fermi_sums(e, n, mu, theta, red);
        mu = mu - 0.1 * (u.f - N);
      }
    }
  }
  // occupations and entropy at the final mu
  double s_entr = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const double s = 1.0 / (1.0 + exp((e[i] - mu) / theta));
    p.occ[(long long)b * n + i] = 2.0 * s;
    s_entr += 2.0 * (xlogx(s) + xlogx(1.0 - s));
  }
  const Sums t = block_sums(s_entr, 0.0, 0.0, red);
  if (threadIdx.x == 0) {
    if (p.mu_out) p.mu_out[b] = mu;
    if (p.entr) p.entr[b] = theta * t.f;
    if (p.loss) p.loss[b] = loss;
    if (p.status) p.status[b] = st;
  }
}

}  // namespace

extern "C" int qex_td_fermi_occupations(int32_t batch, int32_t n, const double* mo_energy,
                                        const double* n_electrons, double theta,
                                        const double* mu_initial, double mu_shift,
                                        double step_grad, int32_t max_steps, int32_t mode,
                                        double* occ, double* mu, double* entropic_energy,
                                        double* loss, int32_t* status, void* stream) {
  if (batch < 0 || n < 1 || !mo_energy || !n_electrons || !occ || !(theta > 0.0) ||
      max_steps < 0 || mode < 0 || mode > 2)
    return QEX_BAD_ARG;
  if (batch == 0) return QEX_OK;
  FermiParams P{batch,   n,   mo_energy, n_electrons,     theta, mu_initial, mu_shift, step_grad,
                max_steps, mode, occ, mu, entropic_energy, loss, status};
  fermi_kernel<<<batch, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(P);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}
