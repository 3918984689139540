// GB300 (sm_103a) 1D Kohn-Sham SCF: one warp per molecule, persistent CTAs,
// every SCF iteration inside one kernel launch.
//
// Reference path (qedft, pasqal-io/qex): qedft/train/od/jit_scf.py:14-244 and
// qedft/train/od/scf.py:32-560 together with the jax_dft primitives they call
// (kinetic matrix, Hartree convolution, dense eigh, density, energies, linear
// mixing).  The arithmetic per iteration follows qedft/train/od/jit_scf.py:26-77:
//   v_H = Hartree(n); v_xc = XC'(n); v_KS = v_H + v_xc + v_ext;
//   (n_out, sum eps, gap) = lowest eigenpairs of T + diag(v_KS);
//   E = sum eps - <v_KS, n_out> + E_H[n_out] + E_xc[n_out] + <v_ext, n_out>;
// then the mixing / convergence rules of jit_scf.py:177-208 (or scf.py:535-558).
//
// GB300 design (FP64 runs at 1/59 of FP32 on this part):
//  * The dense O(N^3) eigh is replaced by a banded selected-eigenpair solver:
//    FP32 Sturm-count multisection (32 lanes x 2 shifts per pass) brackets the
//    lowest eigenvalues, FP32 shifted inverse iteration gives the vectors, and
//    FP64 Newton refinement (FP64 residual, FP32 LDL^T correction solve) brings
//    each eigenpair to FP64 accuracy with only point-parallel FP64 work and no
//    FP64 division.  Near-degenerate clusters get an FP64 Rayleigh-Ritz.
//  * The exponential Hartree kernel is separable: sum_j n_j r^|i-j| is two
//    linear recurrences, computed as a chunked warp scan in O(N) FP64.
//  * The window-MLP exchange-correlation network runs in FP32 with its weights
//    in the kernel's constant parameter bank (broadcast operands).
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <mutex>
#include <type_traits>

#include "ks1d_common.cuh"
#include "ksr_device.cuh"
#include "nn_device.cuh"
#include "xc_device.cuh"
#include "qex_ks1d.h"

namespace qex {
namespace {

// ---------------------------------------------------------------------------
// Launch parameters (passed by value; lives in the constant parameter bank)
// ---------------------------------------------------------------------------
enum Mode { kModeScf = 0, kModeIteration = 1, kModeNonInteracting = 2 };

struct Params {
  int mode;
  int num_molecules;
  const int32_t* order;
  const int32_t* num_grids;
  const int64_t* grid_offsets;
  const double* grid_start;
  const double* grid_spacing;
  const int32_t* num_electrons;
  const int32_t* num_nuclei;
  const double* locations;
  const double* charges;
  const double* vext_in;
  const double* dens_in;
  int max_nuclei;
  int stencil;
  int interaction;
  double ia, ib;
  int iters;
  double alpha, alpha_decay;
  int mixing;
  double tol;
  int rule;
  int reflect;
  int vext_given;
  int nmax;
  int kmax;
  int mix_slots;
  int xc_kind, xc_conv;
  double xc_a, xc_p, xc_shift, lda_A, lda_kappa;
  const float* ksr_w;  // packed KSR network (device)
  double ksr_lo, ksr_hi;
  int ksr_c;
  int ksr_slot;  // constant-memory slot holding the network for this launch
  // KSR: (slot, iteration) rows of nmax doubles receiving the network's input
  // on the output density; the energies then take E_xc from ksr_energy_kernel
  // (one batched evaluation after the SCF) instead of the SCF kernel.  Null:
  // the SCF kernel evaluates it.
  double* ksr_defer;
  // outputs
  double* o_energy;
  double* o_gap;
  uint8_t* o_conv;
  double* o_dens;
  double* o_vh;
  double* o_vxc;
  double* o_f;
  double* o_final;
  double* o_vext;
  int32_t* o_status;
  int32_t* o_iters;
  int32_t* o_stats;
  long long* o_cycles;
  // adjoint step
  const double* a_gnext;  // packed upstream gradient w.r.t. the mixed output density
  const double* a_genergy;  // (B) upstream gradient w.r.t. this iteration's energy
  double a_alpha;         // mixing factor of this iteration
  double* a_gn;           // packed gradient w.r.t. the input density
  double* a_gtheta;       // (B, 577) parameter gradient, accumulated
  double* o_tee;
  // workspace
  double* ws;
  long long stride;  // doubles per molecule
  long long ruw_doubles;  // leading streamed-solve area of a molecule's workspace
  int planes;             // qex_ks1d_options.solve_planes
  int chunk;              // qex_ks1d_options.solve_chunk (points per ring chunk)
  int* counter;
  MlpParams mlp;
  // window MLP in FP64 (a checking mode): 577 doubles in global memory, and
  // 1 / normalization in FP64; null: the FP32 network of `mlp`
  const double* mlp_w64;
  double mlp_norm_inv64;
  // dense networks (QEX_XC_LOCAL_MLP / GLOBAL_MLP): the network, its shared
  // FP32 floats per warp and 4 nmax-double scratch vectors per slot
  NnNet nn;
  int nn_floats;
  double* nn_ws;
};

// Workspace vectors (each nmax doubles) per molecule.
enum Vec { VN = 0, VEXT, VKS, VNOUT, VH, VXC, VF, VKT, VDIFF };
__host__ __device__ inline long long vec_count(int mix_slots, int kmax) {
  return VDIFF + mix_slots + kmax + 2;  // eigenvectors, H x and the FP64 diagonal
}

// Shared-memory layout of one warp (one molecule in flight).
struct SmemLayout {
  int nstr;        // FP32 per-eigenpair stride (nmax rounded to 32k+1)
  size_t s64a, s64b, f32, ring, small, total;
};

// Rows of the streamed-solve area (whole chunks) and its size in doubles.
__host__ __device__ inline long long ruw_rows(int nmax) {
  return (long long)(nmax + kMaxChunk - 1) / kMaxChunk * kMaxChunk;  // whole chunks of any size
}
__host__ __device__ inline long long ruw_doubles(int nmax, int kmax) {
  return ruw_rows(nmax) * kmax * 3 / 2;  // a float2 and a float per point and eigenpair
}

// resident: the FP32 solve planes live in shared memory (small batches, where
// occupancy is not limited by shared memory) instead of streaming through the ring.
__host__ __device__ inline SmemLayout smem_layout(int nmax, int kmax, bool adjoint = false,
                                                  bool resident = false, int nn_floats = 0,
                                                  int chunk = kChunk) {
  SmemLayout L;
  L.nstr = ((nmax + 31) / 32) * 32 + 1;
  size_t off = 0;
  L.s64a = off;
  off += sizeof(double) * (nmax + 2 * kPad64);
  // the second FP64 staging vector and the shared-memory factor arrays are
  // used by the adjoint's Sternheimer solves only
  L.s64b = off;
  if (adjoint) off += sizeof(double) * (nmax + 2 * kPad64);
  off = (off + 15) & ~(size_t)15;  // float4 ring and RR matrices below
  L.f32 = off;
  size_t xc_floats = 2 * (size_t)(nmax + 2 * kPadMlp) + (size_t)kMlpScratch * kWarp;
  if (ksr_scratch_floats(nmax) > xc_floats) xc_floats = ksr_scratch_floats(nmax);
  if ((size_t)nn_floats > xc_floats) xc_floats = (size_t)nn_floats;
  size_t hart_floats = 2 * (size_t)nmax + 2;  // one FP64 scan vector
  // FP32 diagonal, then the ring of the streamed solves (16-byte aligned)
  const size_t ring_off = ((size_t)L.nstr + 3) / 4 * 4;
  L.ring = L.f32 + sizeof(float) * ring_off;
  size_t eig_floats = ring_off + (size_t)(resident ? ruw_rows(nmax) : kRing * chunk) * kmax * 3;
  size_t f = xc_floats > eig_floats ? xc_floats : eig_floats;
  if (hart_floats > f) f = hart_floats;
  if (adjoint) {
    // Sternheimer factor arrays; two padded FP32 windows + an FP32
    // accumulator + per-lane MLP records
    size_t st = (1 + 3 * (size_t)kmax) * L.nstr;
    if (st > f) f = st;
    size_t adj = 3 * (size_t)(nmax + 2 * kPadMlp) + (size_t)kMlpRec * kWarp;
    if (adj > f) f = adj;
  }
  off += sizeof(float) * f;
  off = (off + 15) & ~(size_t)15;
  L.small = off;
  // lo, hi (float x kMaxBis), sig (float x kSamples), cnt (int x kSamples),
  // theta, resn, eigprev (double x kMaxBis), clus (int x kMaxBis), red (double x 32)
  off += sizeof(float) * kMaxBis * 2 + sizeof(float) * kSamples + sizeof(int) * kSamples;
  off = (off + 7) & ~(size_t)7;
  off += sizeof(double) * kMaxBis * 3 + sizeof(int) * kMaxBis;
  off = (off + 7) & ~(size_t)7;
  off += sizeof(double) * 32 + sizeof(double) * 8;  // red, aux
  off = (off + 15) & ~(size_t)15;
  off += sizeof(float) * kMlpFloats;  // MLP weights
  L.total = (off + 127) & ~(size_t)127;
  return L;
}

struct Smem {
  double* s64a;  // padded FP64 staging (index kPad64 + i)
  double* s64b;
  float* f32;
  float4* ring;
  float* lo;
  float* hi;
  float* sig;
  int* cnt;
  double* theta;
  double* resn;
  double* eigprev;
  int* clus;
  double* red;
  double* aux;
  float* mlpw;
  int nstr;
};

__device__ inline Smem carve(unsigned char* base, const SmemLayout& L) {
  Smem s;
  s.s64a = reinterpret_cast<double*>(base + L.s64a);
  s.s64b = reinterpret_cast<double*>(base + L.s64b);
  s.f32 = reinterpret_cast<float*>(base + L.f32);
  s.ring = reinterpret_cast<float4*>(base + L.ring);
  unsigned char* p = base + L.small;
  s.lo = reinterpret_cast<float*>(p);
  p += sizeof(float) * kMaxBis;
  s.hi = reinterpret_cast<float*>(p);
  p += sizeof(float) * kMaxBis;
  s.sig = reinterpret_cast<float*>(p);
  p += sizeof(float) * kSamples;
  s.cnt = reinterpret_cast<int*>(p);
  p += sizeof(int) * kSamples;
  p = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 7) & ~(uintptr_t)7);
  s.theta = reinterpret_cast<double*>(p);
  p += sizeof(double) * kMaxBis;
  s.resn = reinterpret_cast<double*>(p);
  p += sizeof(double) * kMaxBis;
  s.eigprev = reinterpret_cast<double*>(p);
  p += sizeof(double) * kMaxBis;
  s.clus = reinterpret_cast<int*>(p);
  p += sizeof(int) * kMaxBis;
  p = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 7) & ~(uintptr_t)7);
  s.red = reinterpret_cast<double*>(p);
  p += sizeof(double) * 32;
  s.aux = reinterpret_cast<double*>(p);
  p += sizeof(double) * 8;
  p = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 15) & ~(uintptr_t)15);
  s.mlpw = reinterpret_cast<float*>(p);
  s.nstr = L.nstr;
  return s;
}

// ---------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------
struct Stencil {
  double c0, b1, b2;  // diagonal offset, first and second off-diagonal of T
};
__device__ inline Stencil make_stencil(int stencil, double dx) {
  // T = -1/2 L / dx^2; five-point L = (-1/12, 4/3, -5/2, 4/3, -1/12)
  // (jax_dft discrete_laplacian, used at qedft/train/od/scf.py:185-195).
  double inv = 1.0 / (dx * dx);
  Stencil s;
  if (stencil == 5) {
    s.c0 = 1.25 * inv;
    s.b1 = -(2.0 / 3.0) * inv;
    s.b2 = (1.0 / 24.0) * inv;
  } else {
    s.c0 = inv;
    s.b1 = -0.5 * inv;
    s.b2 = 0.0;
  }
  return s;
}

__device__ inline double interaction_fn(const Params& p, double d) {
  if (p.interaction == QEX_INTERACTION_EXPONENTIAL) return p.ia * exp(-p.ib * fabs(d));
  return 1.0 / sqrt(d * d + p.ia);
}

// Stage a global FP64 vector into a padded shared buffer (zeros outside [0,N)).
__device__ inline void stage64(double* s, const double* g, int N, int lane) {
  // zero padding either side; the interior by asynchronous copies, all in
  // flight at once (one memory latency per vector)
  if (lane < kPad64) {
    s[lane] = 0.0;
    s[N + kPad64 + lane] = 0.0;
  }
#pragma unroll 1
  for (int i = lane; i < N; i += kWarp) cp_async8(s + kPad64 + i, g + i);
  cp_async_commit();
  cp_async_wait<0>();
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Hartree: out_i = dx * sum_j n_j K(x_i - x_j)       (qedft/train/od/scf.py:303-308)
// n is staged in sm.s64a (padded).  Returns sum_i n_i * out_i (warp-uniform).
// ---------------------------------------------------------------------------
__device__ __noinline__ double hartree(const Params& p, int N, double dx, const Smem& sm, double* out,
                          const double* kt, int lane) {
  const double* n = sm.s64a + kPad64;
  double acc_e = 0.0;
  if (p.interaction == QEX_INTERACTION_EXPONENTIAL) {
    // sum_j n_j rho^|i-j| = F_i + B_i - n_i with F_i = n_i + rho F_{i-1},
    // B_i = n_i + rho B_{i+1}: chunked affine scans across the warp.
    const double rho = exp(-p.ib * dx);
    double* fwd = reinterpret_cast<double*>(sm.f32);
    const int C = (N + kWarp - 1) / kWarp;
    const int beg = min(lane * C, N);
    const int end = min(beg + C, N);
    double s = 0.0, f = 1.0;
#pragma unroll 1
    for (int i = beg; i < end; ++i) {
      s = fma(s, rho, n[i]);
      f *= rho;
    }
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
      double s2 = __shfl_up_sync(kFull, s, d);
      double f2 = __shfl_up_sync(kFull, f, d);
      if (lane >= d) {
        s = fma(s2, f, s);
        f *= f2;
      }
    }
    double x = __shfl_up_sync(kFull, s, 1);
    if (lane == 0) x = 0.0;
#pragma unroll 1
    for (int i = beg; i < end; ++i) {
      x = fma(x, rho, n[i]);
      fwd[i] = x;
    }
    s = 0.0;
    f = 1.0;
#pragma unroll 1
    for (int i = end - 1; i >= beg; --i) {
      s = fma(s, rho, n[i]);
      f *= rho;
    }
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
      double s2 = __shfl_down_sync(kFull, s, d);
      double f2 = __shfl_down_sync(kFull, f, d);
      if (lane + d < kWarp) {
        s = fma(s2, f, s);
        f *= f2;
      }
    }
    double y = __shfl_down_sync(kFull, s, 1);
    if (lane == kWarp - 1) y = 0.0;
    const double scale = p.ia * dx;
#pragma unroll 1
    for (int i = end - 1; i >= beg; --i) {
      y = fma(y, rho, n[i]);
      double v = scale * (fwd[i] + y - n[i]);
      out[i] = v;
      acc_e = fma(n[i], v, acc_e);
    }
    __syncwarp();
  } else {
    // General (soft-Coulomb) kernel: direct Toeplitz sum with the kernel row
    // kt[d] = K(d dx) tabulated once per molecule.
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      double v = 0.0;
#pragma unroll 1
      for (int j = 0; j < N; ++j) v = fma(n[j], kt[abs(i - j)], v);
      v *= dx;
      out[i] = v;
      acc_e = fma(n[i], v, acc_e);
    }
    __syncwarp();
  }
  return warp_sum(acc_e);
}

// ---------------------------------------------------------------------------
// Exchange-correlation
// ---------------------------------------------------------------------------
// Flip-average v about the grid centre in place (jax_dft
// jit_scf._flip_and_average_on_center, qedft/train/od/jit_scf.py:76-77).
__device__ inline void flip_avg_global(double* v, int N, int lane) {
  #pragma unroll 1
  for (int i = lane; i < N / 2; i += kWarp) {
    double a = v[i], b = v[N - 1 - i];
    double m = 0.5 * (a + b);
    v[i] = m;
    v[N - 1 - i] = m;
  }
  __syncwarp();
}

// Evaluate the XC functional on the density staged in sm.s64a.
//   want_v: write v_xc to vout (FP64 global);  frec: per-point f record or null.
// Returns E_xc (already multiplied by dx).  With reflect_xc the functional is
// symmetrised (local convention, jax_dft kohn_sham_iteration): the staged
// density must already be flip-averaged; outputs are flip-averaged here.
__device__ __noinline__ double nn_xc(const Params& p, int N, double dx, const Smem& sm,
                                     bool want_v, double* vout, double* frec, bool reflect_xc,
                                     double* nnws, int lane);

// Window MLP on the density staged in sm.s64a: the network input n / norm
// with 8 zeros either side and the v_xc accumulator (one window offset at a
// time: distinct addresses per lane, so no atomics are needed) in the FP32
// area, in the network's arithmetic T.  Returns this lane's share of
// sum f n (local) or sum f (amplitude); vout gets v_xc, frec the values.
template <typename T>
__device__ inline double mlp_xc(const Params& p, const T* W, T ninv, int N, double dx,
                                const Smem& sm, bool want_v, double* vout, double* frec,
                                int lane) {
  const double* n = sm.s64a + kPad64;
  const bool local = (p.xc_conv == QEX_XC_LOCAL);
  double e = 0.0;
  T* n32 = reinterpret_cast<T*>(sm.f32);
  T* vacc = n32 + (p.nmax + 2 * kPadMlp);
  #pragma unroll 1
  for (int i = lane; i < N + 2 * kPadMlp; i += kWarp) {
    int k = i - kPadMlp;
    n32[i] = (k >= 0 && k < N) ? (T)n[k] * ninv : T(0);
    vacc[i] = T(0);
  }
  __syncwarp();
  T* scr = vacc + (p.nmax + 2 * kPadMlp) + lane;  // per-lane MLP scratch, stride 32
  const int rounds = (N + kWarp - 1) / kWarp;
  for (int r = 0; r < rounds; ++r) {
    const int i = r * kWarp + lane;
    const bool act = i < N;
    // inactive lanes evaluate a harmless all-zero window
    const T* win = act ? (n32 + i) : (n32 + N + kPadMlp);
    T f;
    if (want_v) {
      f = mlp_point<true>(W, win, act ? 1 : 0, scr, kWarp);
    } else {
      f = mlp_point<false>(W, win, act ? 1 : 0, scr, kWarp);
    }
    double ni = act ? n[i] : 0.0;
    if (act) {
      if (local) {
        e = fma((double)f, ni, e);
      } else {
        e += (double)f;
      }
      if (frec) frec[i] = (double)f;
    }
    if (want_v) {
      const T up = local ? (T)ni * ninv : ninv;
      __syncwarp();
      for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
        if (act) vacc[i + k] += up * scr[k * kWarp];
        __syncwarp();
      }
      if (act && local) vacc[i + kPadMlp] += f;
      __syncwarp();
    }
  }
  if (want_v) {
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      double v = (double)vacc[i + kPadMlp];
      vout[i] = local ? v : dx * v;
    }
  }
  return e;
}

// The FP64 network (checking mode), out of line: its registers stay off the
// FP32 path's.
__device__ __noinline__ double mlp_xc64(const Params& p, int N, double dx, const Smem& sm,
                                        bool want_v, double* vout, double* frec, int lane) {
  return mlp_xc<double>(p, p.mlp_w64, p.mlp_norm_inv64, N, dx, sm, want_v, vout, frec, lane);
}


__device__ __noinline__ double xc_eval(const Params& p, int N, double dx, const Smem& sm, bool want_v,
                          double* vout, double* frec, bool reflect_xc, int lane,
                          double* nnws = nullptr) {
  if (p.xc_kind == QEX_XC_LOCAL_MLP || p.xc_kind == QEX_XC_GLOBAL_MLP)
    return nn_xc(p, N, dx, sm, want_v, vout, frec, reflect_xc, nnws, lane);
  const double* n = sm.s64a + kPad64;
  const bool local = (p.xc_conv == QEX_XC_LOCAL);
  double e = 0.0;
  if (p.xc_kind == QEX_XC_NONE) {
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      if (want_v) vout[i] = 0.0;
      if (frec) frec[i] = 0.0;
    }
    __syncwarp();
    return 0.0;
  }
  if (p.xc_kind == QEX_XC_LDA_EXP_COULOMB || p.xc_kind == QEX_XC_POWER) {
    const LdaConsts lc = lda_consts(p.lda_A, p.lda_kappa);
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      double ni = n[i], f, df = 0.0;
      if (p.xc_kind == QEX_XC_LDA_EXP_COULOMB) {
        if (want_v) {
          lda_exp_coulomb<true>(ni, lc, f, df);
        } else {
          lda_exp_coulomb<false>(ni, lc, f, df);
        }
      } else {
        double base = ni + p.xc_shift;
        f = p.xc_a * pow(base, p.xc_p);
        if (want_v) df = p.xc_a * p.xc_p * pow(base, p.xc_p - 1.0);
      }
      if (local) {
        e = fma(f, ni, e);
        if (want_v) vout[i] = fma(ni, df, f);
      } else {
        e += f;
        if (want_v) vout[i] = dx * df;
      }
      if (frec) frec[i] = f;
    }
  } else {
    e = p.mlp_w64 ? mlp_xc64(p, N, dx, sm, want_v, vout, frec, lane)
                  : mlp_xc<float>(p, sm.mlpw, p.mlp.norm_inv, N, dx, sm, want_v, vout, frec, lane);
  }
  __syncwarp();
  if (reflect_xc) {
    if (want_v) flip_avg_global(vout, N, lane);
    if (frec) flip_avg_global(frec, N, lane);
  }
  return warp_sum(e) * dx;
}

// The dense networks (LocalMLP / GlobalMLP with their wrappers) on the
// density staged in sm.s64a; FP32 network in sm.f32, four scratch vectors of
// nmax doubles at nnws.  Same contract as xc_eval.
__device__ __noinline__ double nn_xc(const Params& p, int N, double dx, const Smem& sm,
                                     bool want_v, double* vout, double* frec, bool reflect_xc,
                                     double* nnws, int lane) {
  const double* n = sm.s64a + kPad64;
  const bool local = (p.xc_conv == QEX_XC_LOCAL);
  double* g = nnws;
  double* gp = nnws + p.nmax;
  double* vs = nnws + 2LL * p.nmax;
  double* c = nnws + 3LL * p.nmax;
  const double e = nn_xc_eval(p.nn, p.xc_kind, N, dx, local, n, want_v, vout, frec, sm.f32, g,
                              gp, vs, c, lane);
  __syncwarp();
  if (reflect_xc) {
    if (want_v) flip_avg_global(vout, N, lane);
    if (frec) flip_avg_global(frec, N, lane);
  }
  return e;
}

// The KSR functional's counterpart of xc_eval, called from the kernel body
// directly: its register footprint then does not add to xc_eval's at the
// other functionals' call sites.
__device__ __noinline__ double ksr_xc(const Params& p, int N, double dx, const Smem& sm,
                                      bool want_v, double* vout, double* frec, bool reflect_xc,
                                      int lane) {
  const double* n = sm.s64a + kPad64;
  const bool local = (p.xc_conv == QEX_XC_LOCAL);
  double e;
  if (p.ksr_c == 16) {
    e = want_v ? ksr_eval<16, true, 1>(p.ksr_w, p.ksr_slot, p.ksr_lo, p.ksr_hi, N, dx, n, local,
                                    vout, frec, sm.f32, lane)
               : ksr_eval<16, false, 1>(p.ksr_w, p.ksr_slot, p.ksr_lo, p.ksr_hi, N, dx, n, local,
                                     nullptr, frec, sm.f32, lane);
  } else {
    e = want_v ? ksr_eval<8, true, 1>(p.ksr_w, p.ksr_slot, p.ksr_lo, p.ksr_hi, N, dx, n, local,
                                   vout, frec, sm.f32, lane)
               : ksr_eval<8, false, 1>(p.ksr_w, p.ksr_slot, p.ksr_lo, p.ksr_hi, N, dx, n, local,
                                    nullptr, frec, sm.f32, lane);
  }
  __syncwarp();
  if (reflect_xc) {
    if (want_v) flip_avg_global(vout, N, lane);
    if (frec) flip_avg_global(frec, N, lane);
  }
  return warp_sum(e) * dx;
}

// ---------------------------------------------------------------------------
// Banded selected-eigenpair solver
// ---------------------------------------------------------------------------
__device__ inline float pseudo_random(int i, int j) {
  unsigned h = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
  h ^= h >> 15;
  h *= 2246822519u;
  h ^= h >> 13;
  return 0.1f + (float)(h & 0xffffu) * (1.0f / 65536.0f) - 0.5f;
}

// FP32 Sturm counts (inertia of L D L^T of H - sigma) for kShiftsPerLane shifts.
template <int kBand>
__device__ inline void sturm_counts(const float* a32, int N, float b1, float b2, float pivmin,
                                    const float* sig, int* cnt) {
  float r1[kShiftsPerLane], r2[kShiftsPerLane], u1[kShiftsPerLane];
  int c[kShiftsPerLane];
#pragma unroll
  for (int s = 0; s < kShiftsPerLane; ++s) {
    r1[s] = 0.0f;
    r2[s] = 0.0f;
    u1[s] = 0.0f;
    c[s] = 0;
  }
  const float b2sq = b2 * b2;
#pragma unroll 2
  for (int i = 0; i < N; ++i) {
    const float a = a32[i];
#pragma unroll
    for (int s = 0; s < kShiftsPerLane; ++s) {
      float d;
      if (kBand == 2) {
        float t = fmaf(-b2, u1[s], b1);
        float u = t * r1[s];
        d = fmaf(-u, t, a - sig[s]);
        d = fmaf(-b2sq, r2[s], d);
        u1[s] = u;
        r2[s] = r1[s];
      } else {
        d = fmaf(-b1 * b1, r1[s], a - sig[s]);
      }
      if (fabsf(d) < pivmin) d = -pivmin;
      c[s] += (d < 0.0f);
      r1[s] = __fdividef(1.0f, d);
    }
  }
#pragma unroll
  for (int s = 0; s < kShiftsPerLane; ++s) cnt[s] = c[s];
}

// L D L^T factorization of H32 - sigma (FP32), stored as r = 1/d and u.
template <int kBand>
__device__ inline void ldl_factor(const float* a32, int N, float b1, float b2, float sigma,
                                  float pivmin, float* R, float* U) {
  float r1 = 0.0f, r2 = 0.0f, u1 = 0.0f;
  const float b2sq = b2 * b2;
#pragma unroll 2
  for (int i = 0; i < N; ++i) {
    float d, u = 0.0f;
    if (kBand == 2) {
      float t = fmaf(-b2, u1, b1);
      u = t * r1;
      d = fmaf(-u, t, a32[i] - sigma);
      d = fmaf(-b2sq, r2, d);
    } else {
      u = b1 * r1;
      d = fmaf(-u, b1, a32[i] - sigma);
    }
    if (fabsf(d) < pivmin) d = (d < 0.0f) ? -pivmin : pivmin;
    float r = __fdividef(1.0f, d);
    R[i] = r;
    U[i] = u;
    r2 = r1;
    r1 = r;
    u1 = u;
  }
}

// Solve (L D L^T) y = scale * x in place in W; returns max |y|.
template <int kBand>
__device__ inline float ldl_solve(int N, float b2, const float* R, const float* U, float* W,
                                  float scale) {
  // Branch-free sweeps: the couplings that reach outside [0, N) multiply a
  // zero carry (z2, y1, y2 start at 0), so they read a clamped in-range index.
  float z1 = 0.0f, z2 = 0.0f;
#pragma unroll 4
  for (int i = 0; i < N; ++i) {
    float z = fmaf(-U[i], z1, W[i] * scale);
    if (kBand == 2) z = fmaf(-b2 * R[max(i - 2, 0)], z2, z);
    W[i] = z * R[i];
    z2 = z1;
    z1 = z;
  }
  float y1 = 0.0f, y2 = 0.0f, mx = 0.0f;
#pragma unroll 4
  for (int i = N - 1; i >= 0; --i) {
    float y = fmaf(-U[min(i + 1, N - 1)], y1, W[i]);
    if (kBand == 2) y = fmaf(-b2 * R[i], y2, y);
    W[i] = y;
    mx = fmaxf(mx, fabsf(y));
    y2 = y1;
    y1 = y;
  }
  return mx;
}

// ---------------------------------------------------------------------------
// Streamed FP32 solves.  The factors and iterates of the K shifted systems live
// in global workspace in two planes with point-major rows of kmax entries: RU
// (float2 {r = 1/d_i, u_i}) and W (the right-hand side / solution w_i).  They
// pass through a ring of kRing chunks of `chunk` points in shared memory
// (cp.async, kRing - 1 chunks in flight), so that the shared-memory footprint
// of a warp does not grow with N * K.
// ---------------------------------------------------------------------------

// The two planes of a molecule's solve area (rows = ruw_rows(nmax)).
struct SolveArea {
  float2* ru;
  float* w;
  int kmax;
  int chunk;  // points per chunk of the ring (streamed planes)
  __device__ float& at(int i, int j) const { return w[(size_t)i * kmax + j]; }
};

// One sweep over points 0..N-1 (kFwd) or N-1..0: lanes with act call
// step(i, ru, w) in order on their own entries (in shared memory); the chunk's
// W entries (and RU with kStoreRU) are then written back.  RU is read only
// with kLoadRU.  The area holds whole chunks, so every copy is in bounds.
template <bool kFwd, bool kLoadRU, bool kStoreRU, bool kRes, typename Step>
__device__ __noinline__ Step ring_sweep(SolveArea g, int N, bool act, float4* ring, int lane,
                                        Step step) {
  const int kmax = g.kmax;
  if (kRes) {
    // planes resident in shared memory: sweep them in place
    if (act) {
      float2* rs = g.ru + lane;
      float* ws = g.w + lane;
      if (kFwd) {
#pragma unroll 4
        for (int i = 0; i < N; ++i) step(i, rs[(size_t)i * kmax], ws[(size_t)i * kmax]);
      } else {
#pragma unroll 4
        for (int i = N - 1; i >= 0; --i) step(i, rs[(size_t)i * kmax], ws[(size_t)i * kmax]);
      }
    }
    __syncwarp();
    return step;
  }
  const int chunk = g.chunk;
  const int nc = (N + chunk - 1) / chunk;
  const int per = chunk * kmax;             // entries per chunk
  const int ru16 = per / 2, w16 = per / 4;  // 16-byte pieces per chunk and plane
  float2* rring = reinterpret_cast<float2*>(ring);
  float* wring = reinterpret_cast<float*>(rring + (size_t)kRing * per);
  auto issue = [&](int k) {
    if (k < nc) {
      const int c = kFwd ? k : nc - 1 - k;
      const int s = k % kRing;
      if (kLoadRU) {
        const float4* src = reinterpret_cast<const float4*>(g.ru + (size_t)c * per);
        float4* dst = reinterpret_cast<float4*>(rring + (size_t)s * per);
#pragma unroll 1
        for (int e = lane; e < ru16; e += kWarp) cp_async16(dst + e, src + e);
      }
      const float4* src = reinterpret_cast<const float4*>(g.w + (size_t)c * per);
      float4* dst = reinterpret_cast<float4*>(wring + (size_t)s * per);
#pragma unroll 1
      for (int e = lane; e < w16; e += kWarp) cp_async16(dst + e, src + e);
    }
    cp_async_commit();
  };
#pragma unroll 1
  for (int k = 0; k < kRing - 1; ++k) issue(k);
#pragma unroll 1
  for (int k = 0; k < nc; ++k) {
    cp_async_wait<kRing - 2>();
    __syncwarp();
    const int s = k % kRing;
    float2* rs = rring + (size_t)s * per + lane;
    float* ws = wring + (size_t)s * per + lane;
    const int c = kFwd ? k : nc - 1 - k;
    const int i0 = c * chunk;
    const int n = min(chunk, N - i0);
    if (act) {
      if (kFwd) {
#pragma unroll 4
        for (int ii = 0; ii < n; ++ii) step(i0 + ii, rs[ii * kmax], ws[ii * kmax]);
      } else {
#pragma unroll 4
        for (int ii = n - 1; ii >= 0; --ii) step(i0 + ii, rs[ii * kmax], ws[ii * kmax]);
      }
    }
    __syncwarp();
    if (kStoreRU) {
      float4* dst = reinterpret_cast<float4*>(g.ru + (size_t)c * per);
      const float4* src = reinterpret_cast<const float4*>(rring + (size_t)s * per);
#pragma unroll 1
      for (int e = lane; e < ru16; e += kWarp) dst[e] = src[e];
    }
    {
      float4* dst = reinterpret_cast<float4*>(g.w + (size_t)c * per);
      const float4* src = reinterpret_cast<const float4*>(wring + (size_t)s * per);
#pragma unroll 1
      for (int e = lane; e < w16; e += kWarp) dst[e] = src[e];
    }
    __syncwarp();
    issue(k + kRing - 1);
  }
  cp_async_wait<0>();
  __syncwarp();
  return step;
}

__device__ inline SolveArea solve_area(double* base, int nmax, int kmax, int chunk) {
  SolveArea a;
  a.ru = reinterpret_cast<float2*>(base);
  a.w = reinterpret_cast<float*>(a.ru + ruw_rows(nmax) * kmax);
  a.kmax = kmax;
  a.chunk = chunk;
  return a;
}

// L D L^T factorisation of H32 - sigma fused with the forward substitution
// L z = w (w overwritten by D^-1 z).
template <int kBand>
struct FactorForward {
  const float* a32;
  float b1, b2, sigma, pivmin;
  float r1 = 0.0f, r2 = 0.0f, u1 = 0.0f, z1 = 0.0f, z2 = 0.0f;
  __device__ void operator()(int i, float2& ru, float& w) {
    float d, u;
    if (kBand == 2) {
      const float t = fmaf(-b2, u1, b1);
      u = t * r1;
      d = fmaf(-u, t, a32[i] - sigma);
      d = fmaf(-b2 * b2, r2, d);
    } else {
      u = b1 * r1;
      d = fmaf(-u, b1, a32[i] - sigma);
    }
    if (fabsf(d) < pivmin) d = (d < 0.0f) ? -pivmin : pivmin;
    const float r = __fdividef(1.0f, d);
    float z = fmaf(-u, z1, w);
    if (kBand == 2) z = fmaf(-b2 * r2, z2, z);
    ru = make_float2(r, u);
    w = z * r;
    r2 = r1;
    r1 = r;
    u1 = u;
    z2 = z1;
    z1 = z;
  }
};

// Forward substitution with stored factors: w <- D^-1 L^-1 (scale w).
template <int kBand>
struct SolveForward {
  float b2, scale;
  float r1 = 0.0f, r2 = 0.0f, z1 = 0.0f, z2 = 0.0f;
  __device__ void operator()(int, float2& ru, float& w) {
    float z = fmaf(-ru.y, z1, w * scale);
    if (kBand == 2) z = fmaf(-b2 * r2, z2, z);
    w = z * ru.x;
    r2 = r1;
    r1 = ru.x;
    z2 = z1;
    z1 = z;
  }
};

// Back substitution L^T y = w in place; tracks max |y|.
template <int kBand>
struct SolveBackward {
  float b2;
  float un = 0.0f, y1 = 0.0f, y2 = 0.0f, mx = 0.0f;
  __device__ void operator()(int, float2& ru, float& w) {
    float y = fmaf(-un, y1, w);
    if (kBand == 2) y = fmaf(-b2 * ru.x, y2, y);
    w = y;
    mx = fmaxf(mx, fabsf(y));
    y2 = y1;
    y1 = y;
    un = ru.y;
  }
};

// Work counters of one eigen-solve (for the roofline tally of the benchmark).
struct EigStats {
  int solves, rq_vectors, updates, passes, fast, fastfail;
  long long cyc[kPhases];  // clock64 cycles per phase (see write_stats)
};

// Adds the cycles since t to phase k and restarts t.
__device__ inline void lap(EigStats& e, long long& t, int k) {
  const long long now = clock64();
  e.cyc[k] += now - t;
  t = now;
}

// Rayleigh-Ritz inside each near-degenerate cluster of eigenpairs (FP64):
// Gram-Schmidt, projected matrix, cyclic Jacobi with the rotations applied to
// the vectors directly, ascending order.  Updates X and sm.theta.
template <int kBand>
__device__ __noinline__ void cluster_rayleigh_ritz(const Params& p, int N, int K, const Stencil& st,
                                                   const double* vks, double* X, double* YR,
                                                   const Smem& sm, int lane) {
  const double* xs = sm.s64a + kPad64;

      int j0 = 0;
      while (j0 < K) {
        int j1 = j0;
        while (j1 + 1 < K && sm.clus[j1 + 1] == sm.clus[j0]) ++j1;
        const int s = j1 - j0 + 1;
        if (s >= 2) {
          for (int a = j0; a <= j1; ++a) {
            double* Xa = X + (size_t)a * p.nmax;
            for (int b = j0; b < a; ++b) {
              const double* Xb = X + (size_t)b * p.nmax;
              double d = 0.0;
              #pragma unroll 1
              for (int i = lane; i < N; i += kWarp) d = fma(Xa[i], Xb[i], d);
              d = warp_sum(d);
              #pragma unroll 1
              for (int i = lane; i < N; i += kWarp) Xa[i] = fma(-d, Xb[i], Xa[i]);
              __syncwarp();
            }
            double nn = 0.0;
            #pragma unroll 1
            for (int i = lane; i < N; i += kWarp) nn = fma(Xa[i], Xa[i], nn);
            nn = warp_sum(nn);
            double inv = 1.0 / sqrt(nn);
            #pragma unroll 1
            for (int i = lane; i < N; i += kWarp) Xa[i] *= inv;
            __syncwarp();
          }
          // projected matrix in the (free) FP32 work area, 16-byte aligned
          double* A = reinterpret_cast<double*>(sm.f32);
          for (int b = j0; b <= j1; ++b) {
            stage64(sm.s64a, X + (size_t)b * p.nmax, N, lane);
            #pragma unroll 1
            for (int i = lane; i < N; i += kWarp) {
              double y = fma(st.c0 + vks[i], xs[i], st.b1 * (xs[i - 1] + xs[i + 1]));
              if (kBand == 2) y = fma(st.b2, xs[i - 2] + xs[i + 2], y);
              YR[i] = y;
            }
            __syncwarp();
            for (int a = j0; a <= b; ++a) {
              const double* Xa = X + (size_t)a * p.nmax;
              double d = 0.0;
              #pragma unroll 1
              for (int i = lane; i < N; i += kWarp) d = fma(Xa[i], YR[i], d);
              d = warp_sum(d);
              if (lane == 0) {
                A[(a - j0) * s + (b - j0)] = d;
                A[(b - j0) * s + (a - j0)] = d;
              }
            }
            __syncwarp();
          }
          for (int sweep = 0; sweep < 30; ++sweep) {
            if (lane == 0) {
              double off = 0.0, dia = 0.0;
              for (int a = 0; a < s; ++a) {
                dia += A[a * s + a] * A[a * s + a];
                for (int b = a + 1; b < s; ++b) off += A[a * s + b] * A[a * s + b];
              }
              sm.aux[2] = (off <= 1e-30 * (1.0 + dia)) ? 1.0 : 0.0;
            }
            __syncwarp();
            if (sm.aux[2] != 0.0) break;
            for (int a = 0; a < s; ++a) {
              for (int b = a + 1; b < s; ++b) {
                if (lane == 0) {
                  double apq = A[a * s + b], c = 1.0, sn = 0.0;
                  if (fabs(apq) > 1e-300) {
                    double app = A[a * s + a], aqq = A[b * s + b];
                    double tau2 = (aqq - app) / (2.0 * apq);
                    double t = (tau2 >= 0 ? 1.0 : -1.0) / (fabs(tau2) + sqrt(1.0 + tau2 * tau2));
                    c = 1.0 / sqrt(1.0 + t * t);
                    sn = t * c;
                    for (int k = 0; k < s; ++k) {
                      double akp = A[k * s + a], akq = A[k * s + b];
                      A[k * s + a] = c * akp - sn * akq;
                      A[k * s + b] = sn * akp + c * akq;
                    }
                    for (int k = 0; k < s; ++k) {
                      double apk = A[a * s + k], aqk = A[b * s + k];
                      A[a * s + k] = c * apk - sn * aqk;
                      A[b * s + k] = sn * apk + c * aqk;
                    }
                  }
                  sm.aux[3] = c;
                  sm.aux[4] = sn;
                }
                __syncwarp();
                const double c = sm.aux[3], sn = sm.aux[4];
                if (sn != 0.0) {
                  double* Xa = X + (size_t)(j0 + a) * p.nmax;
                  double* Xb = X + (size_t)(j0 + b) * p.nmax;
                  #pragma unroll 1
                  for (int i = lane; i < N; i += kWarp) {
                    double xa = Xa[i], xb = Xb[i];
                    Xa[i] = c * xa - sn * xb;
                    Xb[i] = sn * xa + c * xb;
                  }
                }
                __syncwarp();
              }
            }
          }
          // ascending order (swap vectors along with the diagonal)
          for (int a = 0; a < s; ++a) {
            if (lane == 0) {
              int m = a;
              for (int b = a + 1; b < s; ++b)
                if (A[b * s + b] < A[m * s + m]) m = b;
              if (m != a) {
                double t = A[a * s + a];
                A[a * s + a] = A[m * s + m];
                A[m * s + m] = t;
              }
              sm.aux[5] = (double)m;
            }
            __syncwarp();
            const int m = (int)sm.aux[5];
            if (m != a) {
              double* Xa = X + (size_t)(j0 + a) * p.nmax;
              double* Xm = X + (size_t)(j0 + m) * p.nmax;
              #pragma unroll 1
              for (int i = lane; i < N; i += kWarp) {
                double t = Xa[i];
                Xa[i] = Xm[i];
                Xm[i] = t;
              }
            }
            __syncwarp();
          }
          if (lane == 0)
            for (int a = 0; a < s; ++a) sm.theta[j0 + a] = A[a * s + a];
          __syncwarp();
        }
        j0 = j1 + 1;
      }
    }

// Lowest K eigenpairs of T + diag(v) (v in global vks).  X: K vectors of
// stride nmax (FP64, global), normalised to sum x^2 = 1 on exit.
// Eigenvalues in sm.theta[0..K); sm.eigprev holds the previous eigenvalues
// (warm-start brackets), sm.aux[0] the drift bound of eigprev[K] and
// sm.aux[1] whether the previous solve found a cluster.
//
// Two routes:
//  * cold: FP32 multisection -> FP32 inverse iteration -> FP64 refinement
//    (Rayleigh-Ritz inside near-degenerate clusters);
//  * fast (warm start, |dv_KS| < kFastGap x the smallest gap, no clusters): the
//    previous eigenvectors go straight into the FP64 refinement, the FP32
//    factorization taken at their FP64 Rayleigh quotients.  Its result is
//    checked against the Weyl bound |lambda_j - lambda_j^prev| <= |dv|; on
//    failure (or a refinement cap) the cold route runs.
template <int kBand, bool kRes>
__device__ __noinline__ int eigen_solve(const Params& p, int N, double dx, int ne, int K, const double* vks,
                           double* X, SolveArea ruw, bool warm, double dv, const Smem& sm,
                           int lane, EigStats& stats) {
  double* YR = X + (size_t)p.kmax * p.nmax;  // H x of the vector being refined
  double* VA = YR + p.nmax;                  // FP64 diagonal of H
  stats.solves += 1;
  long long tph = clock64();
  const Stencil st = make_stencil(p.stencil, dx);
  float* a32 = sm.f32;
  const int Kc = K + 1;

  // --- FP64 and FP32 diagonal, Gershgorin bounds (FP32: they only seed brackets)
  float aminf = 3e38f, amaxf = -3e38f;
#pragma unroll 1
  for (int i = lane; i < N; i += kWarp) {
    const double a = st.c0 + vks[i];
    const float af = (float)a;
    VA[i] = a;
    a32[i] = af;
    aminf = fminf(aminf, af);
    amaxf = fmaxf(amaxf, af);
  }
  const double amin = (double)warp_minf(aminf);
  const double amax = (double)warp_maxf(amaxf);
  const double rad = 2.0 * fabs(st.b1) + 2.0 * fabs(st.b2);
  const double hnorm = fmax(fabs(amin), fabs(amax)) + rad;
  const float tolabs = (float)(4.0 * FLT_EPSILON * hnorm);
  const float pivmin = (float)(1e-20 * hnorm);
  const float glo = (float)(amin - rad) - tolabs;
  const float ghi = (float)(amax + rad) + tolabs;
  const float b1f = (float)st.b1, b2f = (float)st.b2;
  const float tau = fmaxf(1e-3f, 16.0f * tolabs);
  // residual target: 64 ulp of the operator norm (FP64 floor is ~1 ulp * |H|)
  const double thr = 64.0 * DBL_EPSILON * hnorm;
  double* xs = sm.s64a + kPad64;
  __syncwarp();

  bool fast = false;
  if (warm && sm.aux[1] == 0.0) {
    double gmin = 1e300;
    for (int j = 0; j + 1 < K; ++j) gmin = fmin(gmin, sm.eigprev[j + 1] - sm.eigprev[j]);
    gmin = fmin(gmin, sm.eigprev[K] - sm.aux[0] - sm.eigprev[K - 1]);
    fast = (dv < kFastGap * gmin) && (gmin > (double)tau);
  }

  for (int attempt = 0; attempt < 2; ++attempt) {
    int flags = 0;
    bool any_cluster = false;
    if (fast) {
      if (lane <= K) sm.clus[lane] = lane;
      if (lane < K) sm.resn[lane] = sm.eigprev[lane];  // keep the previous eigenvalues
      __syncwarp();
    } else {
      // ---------------- cold route: brackets
      if (lane < Kc) {
        float lo = glo, hi = ghi;
        if (warm) {
          double c = sm.eigprev[lane];
          double w = dv + (lane == K ? sm.aux[0] : 0.0) + 4.0 * tolabs;
          lo = fmaxf(glo, (float)(c - w));
          hi = fminf(ghi, (float)(c + w));
        }
        sm.lo[lane] = lo;
        sm.hi[lane] = hi;
      }
      __syncwarp();
      int pass = 0;
      if (warm) {
        // verify the warm brackets with one pass of counts at both ends
        float sg[kShiftsPerLane];
        int cn[kShiftsPerLane];
#pragma unroll
        for (int s = 0; s < kShiftsPerLane; ++s) {
          int q = lane * kShiftsPerLane + s;
          int j = q >> 1;
          sg[s] = (j < Kc) ? ((q & 1) ? sm.hi[j] : sm.lo[j]) : 0.0f;
        }
        sturm_counts<kBand>(a32, N, b1f, b2f, pivmin, sg, cn);
#pragma unroll
        for (int s = 0; s < kShiftsPerLane; ++s) sm.cnt[lane * kShiftsPerLane + s] = cn[s];
        __syncwarp();
        if (lane < Kc) {
          int clo = sm.cnt[2 * lane], chi = sm.cnt[2 * lane + 1];
          if (clo > lane) sm.lo[lane] = glo;
          if (chi <= lane) sm.hi[lane] = ghi;
        }
        __syncwarp();
        pass = 1;
      }
      // ---------------- multisection
      for (int it = 0; it < kMaxPasses; ++it) {
        bool unres = false;
        if (lane < Kc) {
          float lo = sm.lo[lane], hi = sm.hi[lane];
          float tol = fmaxf(tolabs, 4.0f * FLT_EPSILON * fmaxf(fabsf(lo), fabsf(hi)));
          unres = (hi - lo) > tol;
          if (unres && lane > 0 && sm.lo[lane - 1] == lo && sm.hi[lane - 1] == hi) unres = false;
        }
        unsigned mask = __ballot_sync(kFull, unres);
        if (mask == 0u) {
          bool any = false;
          if (lane < Kc) {
            float lo = sm.lo[lane], hi = sm.hi[lane];
            float tol = fmaxf(tolabs, 4.0f * FLT_EPSILON * fmaxf(fabsf(lo), fabsf(hi)));
            any = (hi - lo) > tol;
          }
          if (__ballot_sync(kFull, any) == 0u) break;
          mask = __ballot_sync(kFull, any);
        }
        ++pass;
        const int u = __popc(mask);
        const int P = kSamples / u;
        float sg[kShiftsPerLane];
        bool valid[kShiftsPerLane];
#pragma unroll
        for (int s = 0; s < kShiftsPerLane; ++s) {
          int q = lane * kShiftsPerLane + s;
          int k = q / P;
          valid[s] = k < u;
          sg[s] = 0.0f;
          if (valid[s]) {
            unsigned m = mask;
            for (int t = 0; t < k; ++t) m &= m - 1;
            int j = __ffs(m) - 1;
            float lo = sm.lo[j], hi = sm.hi[j];
            int pp = q - k * P;
            sg[s] = lo + __fdividef((hi - lo) * (float)(pp + 1), (float)(P + 1));
          }
        }
        int cn[kShiftsPerLane];
        sturm_counts<kBand>(a32, N, b1f, b2f, pivmin, sg, cn);
        __syncwarp();
#pragma unroll
        for (int s = 0; s < kShiftsPerLane; ++s) {
          int q = lane * kShiftsPerLane + s;
          sm.sig[q] = sg[s];
          sm.cnt[q] = valid[s] ? cn[s] : -1;
        }
        __syncwarp();
        if (lane < Kc) {
          float lo = sm.lo[lane], hi = sm.hi[lane];
          for (int q = 0; q < kSamples; ++q) {
            int c = sm.cnt[q];
            if (c < 0) continue;
            float s = sm.sig[q];
            if (c > lane) {
              hi = fminf(hi, s);
            } else {
              lo = fmaxf(lo, s);
            }
          }
          sm.lo[lane] = lo;
          sm.hi[lane] = hi;
        }
        __syncwarp();
      }
      stats.passes += pass;
      {
        long long t = clock64();
        stats.cyc[2] += t - tph;
        tph = t;
      }
      // ---------------- shifts, clusters
      if (lane < Kc) sm.eigprev[lane] = 0.5 * ((double)sm.lo[lane] + (double)sm.hi[lane]);
      __syncwarp();
      if (lane == 0) {
        int cid = 0;
        sm.clus[0] = 0;
        for (int j = 1; j < Kc; ++j) {
          if (sm.eigprev[j] - sm.eigprev[j - 1] >= tau) ++cid;
          sm.clus[j] = cid;
        }
        sm.aux[0] = 0.0;
      }
      __syncwarp();
      for (int j = 1; j < K; ++j) any_cluster |= (sm.clus[j] == sm.clus[j - 1]);
      {
        // occupied / unoccupied boundary inside a cluster: the density (odd Ne)
        // or the gap (even Ne) is not determined to better than the cluster width
        const int homo = (ne - 1) / 2, lumo = ne / 2;
        bool deg = (homo != lumo) ? (sm.clus[homo] == sm.clus[lumo])
                                  : ((homo > 0 && sm.clus[homo - 1] == sm.clus[homo]) ||
                                     sm.clus[homo] == sm.clus[homo + 1]);
        deg = deg || (sm.clus[K - 1] == sm.clus[K]);
        if (deg) flags |= QEX_FLAG_DEGENERATE_FRONTIER;
      }
      // ---------------- FP32 factorization and inverse iteration (lane j: pair j)
      long long tsub = clock64();
      for (int j = 0; j < K; ++j) {
        const double* Xj = X + (size_t)j * p.nmax;
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp)
          ruw.at(i, j) = warm ? (float)Xj[i] : pseudo_random(i, j);
      }
      __syncwarp();
      lap(stats, tsub, 8);
      const int rounds = warm ? 2 : 4;
      float scale = 1.0f;
      for (int r = 0; r < rounds; ++r) {
        if (r == 0) {
          ring_sweep<true, false, true, kRes>(
              ruw, N, lane < K, sm.ring, lane,
              FactorForward<kBand>{a32, b1f, b2f, lane < K ? (float)sm.eigprev[lane] : 0.0f,
                                   pivmin});
          lap(stats, tsub, 9);
        } else {
          ring_sweep<true, true, false, kRes>(ruw, N, lane < K, sm.ring, lane,
                                        SolveForward<kBand>{b2f, scale});
        }
        const SolveBackward<kBand> bk = ring_sweep<false, true, false, kRes>(
            ruw, N, lane < K, sm.ring, lane, SolveBackward<kBand>{b2f});
        if (lane < K) scale = (bk.mx > 0.0f) ? __fdividef(1.0f, bk.mx) : 1.0f;
        if (any_cluster) {
          // Gram-Schmidt inside clusters (point-parallel)
          for (int j = 1; j < K; ++j) {
            if (sm.clus[j] != sm.clus[j - 1]) continue;
            float sj = __shfl_sync(kFull, scale, j);
            for (int q = j - 1; q >= 0 && sm.clus[q] == sm.clus[j]; --q) {
              float sq = __shfl_sync(kFull, scale, q);
              double dot = 0.0, nq = 0.0;
              #pragma unroll 1
              for (int i = lane; i < N; i += kWarp) {
                double a = (double)ruw.at(i, q) * sq;
                double b = (double)ruw.at(i, j) * sj;
                dot = fma(a, b, dot);
                nq = fma(a, a, nq);
              }
              dot = warp_sum(dot);
              nq = warp_sum(nq);
              const float c = (nq > 0.0) ? __fdividef((float)dot, (float)nq) : 0.0f;
              #pragma unroll 1
              for (int i = lane; i < N; i += kWarp) {
                float& wj = ruw.at(i, j);
                wj = fmaf(-__fdividef(c * sq, sj), ruw.at(i, q), wj);
              }
              __syncwarp();
            }
          }
        }
      }
      lap(stats, tsub, 10);
      // FP64 vectors, normalised
      for (int j = 0; j < K; ++j) {
        float sj = __shfl_sync(kFull, scale, j);
        double nn = 0.0;
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          double a = (double)ruw.at(i, j) * sj;
          nn = fma(a, a, nn);
        }
        nn = warp_sum(nn);
        const double inv = (nn > 0.0) ? rsqrt_nr(nn) : 0.0;
        double* Xj = X + (size_t)j * p.nmax;
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) Xj[i] = (double)ruw.at(i, j) * sj * inv;
      }
      __syncwarp();
      {
        long long t = clock64();
        stats.cyc[3] += t - tph;
        tph = t;
      }
    }

    // ---------------- FP64 Newton refinement: x <- x + (H32 - sigma)^-1 (theta x - H x)
    bool done_all = false;
    long long tsub = clock64();
    // shift of each lane's current factorisation, and the last residual
    float sig_cur = (!fast && lane < K) ? (float)sm.eigprev[lane] : 0.0f;
    double red_prev = 1e300;
    for (int step = 0; step < kMaxRefineSteps; ++step) {
      stats.rq_vectors += K;
      // Rayleigh quotient and residual of each vector: FP64 H x (the residual
      // cancels to ~1e-14 of |H|), FP32 residual norm (3 digits suffice)
      for (int j = 0; j < K; ++j) {
        stage64(sm.s64a, X + (size_t)j * p.nmax, N, lane);
        double xx = 0.0, xy = 0.0;
#pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          const double x = xs[i];
          double y = fma(VA[i], x, st.b1 * (xs[i - 1] + xs[i + 1]));
          if (kBand == 2) y = fma(st.b2, xs[i - 2] + xs[i + 2], y);
          YR[i] = y;
          xx = fma(x, x, xx);
          xy = fma(x, y, xy);
        }
        warp_sum2(xx, xy, lane);
        const double th = div_nr(xy, xx);
        float rr = 0.0f;
#pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          const float r = (float)fma(-th, xs[i], YR[i]);
          rr = fmaf(r, r, rr);
          ruw.at(i, j) = -r;
        }
        rr = warp_sumf(rr);
        if (lane == 0) {
          sm.theta[j] = th;
          sm.red[j] = (double)sqrtf(__fdividef(rr, (float)xx));
        }
        __syncwarp();
      }
      lap(stats, tsub, 11);
      bool need = false;
      if (lane < K) {
        bool inclus = (lane > 0 && sm.clus[lane] == sm.clus[lane - 1]) ||
                      (lane + 1 < Kc && sm.clus[lane] == sm.clus[lane + 1]);
        need = inclus ? (step < 3) : (sm.red[lane] > thr);
      }
      const unsigned nm = __ballot_sync(kFull, need);
      if (nm == 0u) {
        done_all = true;
        break;
      }
      stats.updates += __popc(nm);
      // factorise at the FP64 Rayleigh quotient on the fast route's first step
      // and wherever the last correction gained less than two digits (a vector
      // that needs no correction now never needs one later)
      const bool refac = need && ((fast && step == 0) || (step > 0 && sm.red[lane] > 1e-2 * red_prev));
      if (lane < K) red_prev = sm.red[lane];
      if (refac) sig_cur = (float)sm.theta[lane];
      if (__any_sync(kFull, refac)) {
        ring_sweep<true, false, true, kRes>(ruw, N, need, sm.ring, lane,
                                      FactorForward<kBand>{a32, b1f, b2f, sig_cur, pivmin});
      } else {
        ring_sweep<true, true, false, kRes>(ruw, N, need, sm.ring, lane, SolveForward<kBand>{b2f, 1.0f});
      }
      ring_sweep<false, true, false, kRes>(ruw, N, need, sm.ring, lane, SolveBackward<kBand>{b2f});
      lap(stats, tsub, 12);
      for (int j = 0; j < K; ++j) {
        if (!((nm >> j) & 1u)) continue;
        double* Xj = X + (size_t)j * p.nmax;
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) Xj[i] += (double)ruw.at(i, j);
      }
      __syncwarp();
      lap(stats, tsub, 13);
    }
    lap(stats, tsub, 11);

    if (fast) {
      stats.fast += 1;
      // Weyl check: each eigenvalue moved by at most |dv| (plus rounding)
      bool ok = done_all;
      if (lane < K) {
        double moved = fabs(sm.theta[lane] - sm.resn[lane]);
        ok = ok && (moved <= dv + 1e-9 * hnorm);
      }
      ok = __all_sync(kFull, ok || lane >= K);
      if (!ok) {
        stats.fastfail += 1;
        // restore the previous eigenvalues as warm brackets and take the cold route
        if (lane < K) sm.eigprev[lane] = sm.resn[lane];
        __syncwarp();
        fast = false;
        {
          long long t = clock64();
          stats.cyc[4] += t - tph;
          tph = t;
        }
        continue;
      }
    }
    if (!done_all) flags |= QEX_FLAG_REFINE_CAP;

    // ---------------- Rayleigh-Ritz inside clusters (FP64); Jacobi rotations
    // are applied to the vectors directly
    tsub = clock64();
    if (any_cluster) cluster_rayleigh_ritz<kBand>(p, N, K, st, vks, X, YR, sm, lane);

    // ---------------- final normalisation and warm-start data
    for (int j = 0; j < K; ++j) {
      double* Xj = X + (size_t)j * p.nmax;
      double nn = 0.0;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) nn = fma(Xj[i], Xj[i], nn);
      nn = warp_sum(nn);
      const double inv = rsqrt_nr(nn);
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) Xj[i] *= inv;
    }
    lap(stats, tsub, 15);
    if (lane < K) sm.eigprev[lane] = sm.theta[lane];
    if (lane == 0) {
      if (fast) sm.aux[0] += dv;  // eigprev[K] is not refreshed on the fast route
      sm.aux[1] = any_cluster ? 1.0 : 0.0;
    }
    __syncwarp();
    stats.cyc[4] += clock64() - tph;
    return flags;
  }
  return QEX_FLAG_REFINE_CAP;
}

// Occupation of orbital j for Ne electrons (two per orbital, last one single
// when Ne is odd: jnp.repeat(..., 2)[:Ne], qedft/train/od/scf.py:212-213).
__device__ inline double occupation(int j, int ne) {
  int rem = ne - 2 * j;
  return rem >= 2 ? 2.0 : (rem == 1 ? 1.0 : 0.0);
}

// Density, eigen-energy sum and gap from the eigenpairs.
__device__ __noinline__ void density_from_orbitals(const Params& p, int N, double dx, int ne, int K,
                                      const double* X, double* nout, const Smem& sm, double& tee,
                                      double& gap, int lane) {
  const int nocc = (ne + 1) / 2;
  const int nfull = ne / 2;  // doubly occupied; with odd ne, orbital nfull holds one
  const double inv_dx = recip_nr(dx);
#pragma unroll 1
  for (int i = lane; i < N; i += kWarp) {
    double v = 0.0;
    for (int j = 0; j < nfull; ++j) {
      const double x = X[(size_t)j * p.nmax + i];
      v = fma(x, x, v);
    }
    v += v;
    if (nfull < nocc) {
      const double x = X[(size_t)nfull * p.nmax + i];
      v = fma(x, x, v);
    }
    nout[i] = v * inv_dx;
  }
  tee = 0.0;
  for (int j = 0; j < nocc; ++j) tee += occupation(j, ne) * sm.theta[j];
  // jax_dft get_gap: repeated spectrum rep[Ne] - rep[Ne-1]
  const int lumo = ne / 2, homo = (ne - 1) / 2;
  gap = sm.theta[lumo] - sm.theta[homo];
  (void)K;
  __syncwarp();
}

__device__ inline void write_stats(const Params& p, int b, const EigStats& e) {
  if (!p.o_stats) return;
  p.o_stats[8 * b + 0] = e.solves;
  p.o_stats[8 * b + 1] = e.rq_vectors;
  p.o_stats[8 * b + 2] = e.updates;
  p.o_stats[8 * b + 3] = e.passes;
  p.o_stats[8 * b + 4] = e.fast;
  p.o_stats[8 * b + 5] = e.fastfail;
  if (p.o_cycles)
    for (int k = 0; k < kPhases; ++k) p.o_cycles[(long long)kPhases * b + k] = e.cyc[k];
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
// kKsr: the KSR functional's instantiation.  Its evaluation needs far more
// registers than the other functionals', and a callee that large anywhere in
// the call graph makes the whole persistent kernel spill, so only this
// instantiation calls it.
template <int kBand, bool kRes, bool kKsr>
__global__ void __launch_bounds__(kWarp, 12) ks1d_kernel(const __grid_constant__ Params p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x;
  const SmemLayout L = smem_layout(p.nmax, p.kmax, false, kRes, p.nn_floats, p.chunk);
  Smem sm = carve(smem_raw, L);
  if (p.xc_kind == QEX_XC_WINDOW_MLP) stage_mlp_weights(p.mlp, sm.mlpw, lane, kWarp);
  __syncwarp();

  for (;;) {
    int slot = 0;
    if (lane == 0) slot = atomicAdd(p.counter, 1);
    slot = __shfl_sync(kFull, slot, 0);
    if (slot >= p.num_molecules) break;
    const int b = p.order ? p.order[slot] : slot;

    const int N = p.num_grids[b];
    const long long off = p.grid_offsets[b];
    const int ne = p.num_electrons[b];
    const double x0 = p.grid_start[b];
    const double dx = p.grid_spacing[b];
    const int K = ne / 2 + 1;
    if (N < 5 || N > p.nmax || ne < 1 || K > p.kmax || !(dx > 0.0) ||
        (p.xc_kind == QEX_XC_GLOBAL_MLP && N != p.nn.inputs)) {
      if (lane == 0 && p.o_status) p.o_status[b] = QEX_BAD_ARG;
      continue;
    }
    double* const slot_base = p.ws + (long long)slot * p.stride;
    const SolveArea ruw = kRes ? solve_area(reinterpret_cast<double*>(sm.ring), p.nmax, p.kmax,
                                            p.chunk)
                               : solve_area(slot_base, p.nmax, p.kmax, p.chunk);  // FP32 solve planes
    double* ws = slot_base + p.ruw_doubles;
    double* vn = ws + (long long)VN * p.nmax;
    double* vext = ws + (long long)VEXT * p.nmax;
    double* vks = ws + (long long)VKS * p.nmax;
    double* nout = ws + (long long)VNOUT * p.nmax;
    double* vh = ws + (long long)VH * p.nmax;
    double* vxc = ws + (long long)VXC * p.nmax;
    double* vf = ws + (long long)VF * p.nmax;
    double* kt = ws + (long long)VKT * p.nmax;
    double* diffs = ws + (long long)VDIFF * p.nmax;
    double* X = diffs + (long long)p.mix_slots * p.nmax;
    double* const nnws = p.nn_ws ? p.nn_ws + 4LL * slot * p.nmax : nullptr;
    int flags = 0;
    EigStats est = {};
    long long tmol = clock64();

    // external potential and interaction table
    if (p.vext_given) {
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) vext[i] = p.vext_in[off + i];
    } else {
      const int M = p.num_nuclei[b];
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        double x = x0 + i * dx, v = 0.0;
        for (int m = 0; m < M; ++m) {
          double R = p.locations[(long long)b * p.max_nuclei + m];
          double Z = p.charges[(long long)b * p.max_nuclei + m];
          v -= Z * interaction_fn(p, x - R);
        }
        vext[i] = v;
      }
    }
    if (p.interaction != QEX_INTERACTION_EXPONENTIAL) {
      #pragma unroll 1
      for (int d = lane; d < N; d += kWarp) kt[d] = interaction_fn(p, d * dx);
    }
    if (p.o_vext)
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) p.o_vext[off + i] = vext[i];
    __syncwarp();

    if (p.mode == kModeNonInteracting) {
      flags |= eigen_solve<kBand, kRes>(p, N, dx, ne, K, vext, X, ruw, false, 0.0, sm, lane, est);
      double tee, gap;
      density_from_orbitals(p, N, dx, ne, K, X, nout, sm, tee, gap, lane);
      if (p.o_final)
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) p.o_final[off + i] = nout[i];
      if (lane == 0) {
        if (p.o_tee) p.o_tee[b] = tee;
        if (p.o_gap) p.o_gap[b] = gap;
        if (p.o_status) p.o_status[b] = flags;
        write_stats(p, b, est);
      }
      continue;
    }

    // initial density
    bool warm = false;
    double dv = 0.0;
    if (p.dens_in) {
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) vn[i] = p.dens_in[off + i];
    } else {
      flags |= eigen_solve<kBand, kRes>(p, N, dx, ne, K, vext, X, ruw, false, 0.0, sm, lane, est);
      double tee, gap;
      density_from_orbitals(p, N, dx, ne, K, X, vn, sm, tee, gap, lane);
      // warm start from the non-interacting eigenpairs: v_KS differs from
      // v_ext by v_H + v_xc, bounded below through dv in the first iteration.
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) vks[i] = vext[i];
      warm = true;
    }
    __syncwarp();

    double alpha = p.alpha;
    bool converged = false;
    int active = 0;
    int last_t = 0;  // last iteration that ran (the converged branch repeats it)
    double last_energy = INFINITY, last_gap = 0.0;
    const long long rec = (long long)p.iters * off;
    const bool reflect_xc = p.reflect && p.xc_conv == QEX_XC_LOCAL;
    const int slots = p.mix_slots;

    for (int t = 0; t < p.iters; ++t) {
      const long long r0 = rec + (long long)t * N;
      if (converged && p.mode == kModeScf) {
        // converged branch: the previous state is repeated (jit_scf.py:164-166,
        // scf.py:522-524)
        if (lane == 0) {
          if (p.o_energy) p.o_energy[(long long)b * p.iters + t] = last_energy;
          if (p.o_gap) p.o_gap[(long long)b * p.iters + t] = last_gap;
          if (p.o_conv) p.o_conv[(long long)b * p.iters + t] = 1;
        }
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          if (p.o_dens) p.o_dens[r0 + i] = vn[i];
          if (p.o_vh) p.o_vh[r0 + i] = vh[i];
          if (p.o_vxc) p.o_vxc[r0 + i] = vxc[i];
          if (p.o_f) p.o_f[r0 + i] = vf[i];
        }
        if constexpr (kKsr) {
          if (p.ksr_defer) {
            const double* src = p.ksr_defer + ((long long)slot * p.iters + last_t) * p.nmax;
            double* dst = p.ksr_defer + ((long long)slot * p.iters + t) * p.nmax;
            #pragma unroll 1
            for (int i = lane; i < N; i += kWarp) dst[i] = src[i];
          }
        }
        continue;
      }
      const bool conv_at_start = converged;
      if (p.mode == kModeIteration) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) vn[i] = p.dens_in[off + i];
        __syncwarp();
      }

      // ---- Hartree and XC on the input density
      long long tit = clock64();
      stage64(sm.s64a, vn, N, lane);
      hartree(p, N, dx, sm, vh, kt, lane);
      {
        long long t = clock64();
        est.cyc[0] += t - tit;
        tit = t;
      }
      if (reflect_xc) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          sm.s64a[kPad64 + i] = 0.5 * (vn[i] + vn[N - 1 - i]);
        }
        __syncwarp();
      }
      if constexpr (kKsr) {
        ksr_xc(p, N, dx, sm, true, vxc, vf, reflect_xc, lane);
      } else {
        xc_eval(p, N, dx, sm, true, vxc, vf, reflect_xc, lane, nnws);
      }
      // |dv_KS|_inf in FP32, rounded up: it only sizes brackets and picks the
      // warm route, both of which are verified
      float dvl = 0.0f;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        double v = vh[i] + vxc[i] + vext[i];
        dvl = fmaxf(dvl, fabsf((float)(v - vks[i])));
        vks[i] = v;
      }
      dv = warm ? (double)warp_maxf(dvl) * (1.0 + 1e-6) : 0.0;
      __syncwarp();
      {
        long long t = clock64();
        est.cyc[1] += t - tit;
      }

      // ---- eigen-solve and output density
      flags |= eigen_solve<kBand, kRes>(p, N, dx, ne, K, vks, X, ruw, warm, dv, sm, lane, est);
      warm = true;
      tit = clock64();
      double tee, gap;
      density_from_orbitals(p, N, dx, ne, K, X, nout, sm, tee, gap, lane);

      // ---- total energy on the output density (jit_scf.py:46-72)
      double eks = 0.0, eext = 0.0;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        eks = fma(vks[i], nout[i], eks);
        eext = fma(vext[i], nout[i], eext);
      }
      eks = warp_sum(eks) * dx;
      eext = warp_sum(eext) * dx;
      stage64(sm.s64a, nout, N, lane);
      // Hartree of n_out into the refinement scratch (only the energy is kept)
      const double eh = 0.5 * dx * hartree(p, N, dx, sm, X + (long long)p.kmax * p.nmax, kt, lane);
      __syncwarp();
      if (reflect_xc) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          sm.s64a[kPad64 + i] = 0.5 * (nout[i] + nout[N - 1 - i]);
        }
        __syncwarp();
      }
      long long tsub = clock64();
      double exc;
      if constexpr (kKsr) {
        if (p.ksr_defer && p.mode == kModeScf) {
          // the network's input, evaluated after the SCF by ksr_energy_kernel
          double* row = p.ksr_defer + ((long long)slot * p.iters + t) * p.nmax;
          #pragma unroll 1
          for (int i = lane; i < N; i += kWarp) row[i] = sm.s64a[kPad64 + i];
          last_t = t;
          exc = 0.0;
        } else {
          exc = ksr_xc(p, N, dx, sm, false, nullptr, nullptr, false, lane);
        }
      } else {
        exc = xc_eval(p, N, dx, sm, false, nullptr, nullptr, false, lane, nnws);
      }
      lap(est, tsub, 14);
      const double energy = tee - eks + eh + exc + eext;
      if (p.reflect) flip_avg_global(nout, N, lane);
      {
        long long t = clock64();
        est.cyc[5] += t - tit;
        tit = t;
      }

      if (p.mode == kModeIteration) {
        if (lane == 0) {
          if (p.o_energy) p.o_energy[b] = energy;
          if (p.o_gap) p.o_gap[b] = gap;
          if (p.o_status) p.o_status[b] = flags;
          if (p.o_iters) p.o_iters[b] = 1;
          write_stats(p, b, est);
        }
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          if (p.o_dens) p.o_dens[off + i] = nout[i];
          if (p.o_vh) p.o_vh[off + i] = vh[i];
          if (p.o_vxc) p.o_vxc[off + i] = vxc[i];
          if (p.o_f) p.o_f[off + i] = vf[i];
          if (p.o_final) p.o_final[off + i] = nout[i];
        }
        break;
      }

      // ---- mixing (jit_scf.py:177-181; scf.py:547-555)
      const int slot_w = active % slots;
      double* dslot = diffs + (long long)slot_w * p.nmax;
      const int navg = min(active + 1, min(p.mixing, slots));
      double mse_raw = 0.0, mse_mix = 0.0;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        double d = nout[i] - vn[i];
        dslot[i] = d;
        mse_raw = fma(d, d, mse_raw);
      }
      __syncwarp();
      const double coef = (navg == 1) ? alpha : div_nr(alpha, (double)navg);
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        double s = 0.0;
        for (int q = 0; q < navg; ++q) {
          int sl = (active - q) % slots;
          if (sl < 0) sl += slots;
          s += diffs[(long long)sl * p.nmax + i];
        }
        const double upd = coef * s;
        mse_mix = fma(upd, upd, mse_mix);
        vn[i] += upd;
      }
      warp_sum2(mse_raw, mse_mix, lane);
      mse_raw = div_nr(mse_raw, (double)N);
      mse_mix = div_nr(mse_mix, (double)N);
      __syncwarp();
      ++active;
      bool rec_conv;
      if (p.rule == 0) {
        rec_conv = conv_at_start;
        converged = mse_mix < p.tol;
        alpha *= p.alpha_decay;
      } else {
        converged = mse_raw < p.tol;
        rec_conv = converged;
        alpha *= p.alpha_decay;
      }
      last_energy = energy;
      last_gap = gap;
      if (lane == 0) {
        if (p.o_energy) p.o_energy[(long long)b * p.iters + t] = energy;
        if (p.o_gap) p.o_gap[(long long)b * p.iters + t] = gap;
        if (p.o_conv) p.o_conv[(long long)b * p.iters + t] = rec_conv ? 1 : 0;
      }
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        if (p.o_dens) p.o_dens[r0 + i] = vn[i];
        if (p.o_vh) p.o_vh[r0 + i] = vh[i];
        if (p.o_vxc) p.o_vxc[r0 + i] = vxc[i];
        if (p.o_f) p.o_f[r0 + i] = vf[i];
      }
      __syncwarp();
      est.cyc[6] += clock64() - tit;
    }
    est.cyc[7] = clock64() - tmol;
    if (p.mode == kModeScf) {
      if (p.o_final)
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) p.o_final[off + i] = vn[i];
      if (lane == 0) {
        if (p.o_status) p.o_status[b] = flags;
        if (p.o_iters) p.o_iters[b] = active;
        write_stats(p, b, est);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Adjoint of one SCF iteration (local convention, window-MLP XC, exponential
// interaction, one mixing difference):
//   n_{t+1} = (1 - a) n_t + a m_t,   m_t = sum_j occ_j phi_j^2 / dx,
//   v_t = v_H(n_t) + v_xc(n_t; theta) + v_ext,   (phi_j, lambda_j) = eig(T + v_t),
//   E_t = sum occ lambda - dx<v_t, m_t> + E_H(m_t) + E_xc(m_t; theta) + dx<v_ext, m_t>.
// Reverse: gm = a gnext + gE dx (v_H(m) + v_xc(m) + v_ext - v_t)   (dE/dv_t = 0),
//   gv = chi gm (static response: Sternheimer solves of (H - lambda_j) y = -Q(phi_j gm)
//   in the unoccupied complement, plus occupied pairs of unequal occupation),
//   gn = (1 - a) gnext + v_H(gv) + d/dn [v_xc(n) . gv],
//   gtheta += gE d/dtheta E_xc(m) + d/dtheta [v_xc(n) . gv].
// ---------------------------------------------------------------------------

// FP64 banded (H - shift) x with x staged in sm.s64a, result in ys.
template <int kBand>
__device__ inline void banded_apply(const Stencil& st, const double* vks, double shift, int N,
                                    const double* xs, double* ys, int lane) {
  #pragma unroll 1
  for (int i = lane; i < N; i += kWarp) {
    double y = fma(st.c0 + vks[i] - shift, xs[i], st.b1 * (xs[i - 1] + xs[i + 1]));
    if (kBand == 2) y = fma(st.b2, xs[i - 2] + xs[i + 2], y);
    ys[i] = y;
  }
  __syncwarp();
}

// v <- v - sum_k (phi_k . v) phi_k over the nocc occupied orbitals (FP64, in place)
__device__ inline void project_out(double* v, const double* X, int nmax, int nocc, int N,
                                   int lane) {
  for (int k = 0; k < nocc; ++k) {
    const double* Xk = X + (size_t)k * nmax;
    double c = 0.0;
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) c = fma(Xk[i], v[i], c);
    c = warp_sum(c);
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) v[i] = fma(-c, Xk[i], v[i]);
    __syncwarp();
  }
}

// gv = chi gm.  Y, Bv: K vectors each (workspace).  Returns the refinement steps used.
template <int kBand>
__device__ int sternheimer(const Params& p, int N, double dx, int ne, const double* vks,
                           const double* X, const double* gm, double* Y, double* Bv, double* gv,
                           const Smem& sm, int lane) {
  const Stencil st = make_stencil(p.stencil, dx);
  const int nocc = (ne + 1) / 2;
  const int nstr = sm.nstr;
  float* a32 = sm.f32;
  float* R = a32 + nstr;
  float* U = R + (size_t)p.kmax * nstr;
  float* W = U + (size_t)p.kmax * nstr;
  double amax = 0.0;
  #pragma unroll 1
  for (int i = lane; i < N; i += kWarp) {
    const double a = st.c0 + vks[i];
    a32[i] = (float)a;
    amax = fmax(amax, fabs(a));
  }
  amax = warp_max(amax);
  const double hnorm = amax + 2.0 * fabs(st.b1) + 2.0 * fabs(st.b2);
  const float pivmin = (float)(1e-20 * hnorm);
  __syncwarp();
  if (lane < nocc)
    ldl_factor<kBand>(a32, N, (float)st.b1, (float)st.b2, (float)sm.theta[lane], pivmin,
                      R + (size_t)lane * nstr, U + (size_t)lane * nstr);
  // right-hand sides b_j = -Q (phi_j gm), y_j = 0
  for (int j = 0; j < nocc; ++j) {
    const double* Xj = X + (size_t)j * p.nmax;
    double* Bj = Bv + (size_t)j * p.nmax;
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      Bj[i] = -Xj[i] * gm[i];
      Y[(size_t)j * p.nmax + i] = 0.0;
    }
    __syncwarp();
    project_out(Bj, X, p.nmax, nocc, N, lane);
  }
  double* xs = sm.s64a + kPad64;
  double* ys = sm.s64b + kPad64;
  int steps = 0;
  for (; steps < 12; ++steps) {
    bool need = false;
    for (int j = 0; j < nocc; ++j) {
      const double* Bj = Bv + (size_t)j * p.nmax;
      stage64(sm.s64a, Y + (size_t)j * p.nmax, N, lane);
      banded_apply<kBand>(st, vks, sm.theta[j], N, xs, ys, lane);
      project_out(ys, X, p.nmax, nocc, N, lane);
      double rr = 0.0, bb = 0.0;
      float* Wj = W + (size_t)j * nstr;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        const double r = Bj[i] - ys[i];
        rr = fma(r, r, rr);
        bb = fma(Bj[i], Bj[i], bb);
        Wj[i] = (float)r;
      }
      rr = warp_sum(rr);
      bb = warp_sum(bb);
      if (lane == j) need = rr > 1e-26 * bb;
      __syncwarp();
    }
    const unsigned nm = __ballot_sync(kFull, need);
    if (nm == 0u) break;
    if (need)
      ldl_solve<kBand>(N, (float)st.b2, R + (size_t)lane * nstr, U + (size_t)lane * nstr,
                       W + (size_t)lane * nstr, 1.0f);
    __syncwarp();
    for (int j = 0; j < nocc; ++j) {
      if (!((nm >> j) & 1u)) continue;
      const float* Wj = W + (size_t)j * nstr;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) ys[i] = (double)Wj[i];
      __syncwarp();
      project_out(ys, X, p.nmax, nocc, N, lane);
      double* Yj = Y + (size_t)j * p.nmax;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) Yj[i] += ys[i];
      __syncwarp();
    }
  }
  // gv = sum_j (2 occ_j / dx) phi_j y_j
  const double inv_dx = 1.0 / dx;
  #pragma unroll 1
  for (int i = lane; i < N; i += kWarp) {
    double v = 0.0;
    for (int j = 0; j < nocc; ++j)
      v = fma(2.0 * occupation(j, ne) * inv_dx * X[(size_t)j * p.nmax + i], Y[(size_t)j * p.nmax + i], v);
    gv[i] = v;
  }
  __syncwarp();
  // occupied pairs of unequal occupation (the half-filled HOMO of odd Ne)
  if (ne & 1) {
    const int h = nocc - 1;
    const double* Xh = X + (size_t)h * p.nmax;
    for (int k = 0; k < h; ++k) {
      const double* Xk = X + (size_t)k * p.nmax;
      double c = 0.0;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) c = fma(Xk[i] * Xh[i], gm[i], c);
      c = warp_sum(c);
      const double f = 2.0 * inv_dx * (occupation(h, ne) - occupation(k, ne)) /
                       (sm.theta[h] - sm.theta[k]) * c;
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) gv[i] = fma(f * Xh[i], Xk[i], gv[i]);
      __syncwarp();
    }
  }
  return steps;
}

// One MLP pass for the adjoint over all points of the molecule.
//   n32 / u32: padded FP32 windows (density / norm, direction / norm)
//   ybar_i = ya[i] * yscale, dybar_i = with_tangent ? n[i] : 0
//   xbar scattered into gacc (FP32, padded), dy added to gn (FP64) if with_tangent.
template <typename T>
__device__ void mlp_adjoint_pass(const T* W, T ninv, int N, const T* n32, const T* u32,
                                 bool with_tangent, const double* ya, double yscale,
                                 const double* nvec, T* gacc, double* gn, T* rec, double* acc,
                                 int lane) {
  const int rounds = (N + kWarp - 1) / kWarp;
  const T* zero_win = n32 + N + kPadMlp;  // 8+ zeros
  for (int r = 0; r < rounds; ++r) {
    const int i = r * kWarp + lane;
    const bool act = i < N;
    const T* win = act ? (n32 + i) : zero_win;
    const T* twin = (act && with_tangent) ? (u32 + i) : zero_win;
    // inactive lanes (and the tangent of a pass without one) read a single
    // zero element with stride 0
    const int stride = act ? 1 : 0;
    const int tstride = (act && with_tangent) ? 1 : 0;
    const T ybar = act ? (T)(ya[i] * yscale) : T(0);
    const T dybar = (act && with_tangent) ? (T)nvec[i] : T(0);
    const T dy = mlp_dual_reverse(W, win, stride, twin, tstride, ybar, dybar, rec + lane, kWarp);
    __syncwarp();
    mlp_param_grad_round(rec, lane, acc);
    for (int k = 0; k < QEX_MLP_WINDOW; ++k) {
      if (act) gacc[i + k] += rec[(147 + k) * kWarp + lane] * ninv;
      __syncwarp();
    }
    if (act && with_tangent) gn[i] += (double)dy;
    __syncwarp();
  }
}

template <int kBand, bool kNet64>
__global__ void __launch_bounds__(kWarp, 8) ks1d_adjoint_kernel(const __grid_constant__ Params p) {
  using T = typename std::conditional<kNet64, double, float>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x;
  const SmemLayout L = smem_layout(p.nmax, p.kmax, true, false, p.nn_floats, p.chunk);
  Smem sm = carve(smem_raw, L);
  stage_mlp_weights(p.mlp, sm.mlpw, lane, kWarp);
  __syncwarp();
  const int slots = p.mix_slots;
  for (;;) {
    int slot = 0;
    if (lane == 0) slot = atomicAdd(p.counter, 1);
    slot = __shfl_sync(kFull, slot, 0);
    if (slot >= p.num_molecules) break;
    const int b = p.order ? p.order[slot] : slot;
    const int N = p.num_grids[b];
    const long long off = p.grid_offsets[b];
    const int ne = p.num_electrons[b];
    const double x0 = p.grid_start[b];
    const double dx = p.grid_spacing[b];
    const int K = ne / 2 + 1;
    if (N < 5 || N > p.nmax || ne < 1 || K > p.kmax || !(dx > 0.0)) {
      if (lane == 0 && p.o_status) p.o_status[b] = QEX_BAD_ARG;
      continue;
    }
    double* const slot_base = p.ws + (long long)slot * p.stride;
    const SolveArea ruw = solve_area(slot_base, p.nmax, p.kmax, p.chunk);  // streamed FP32 solves
    double* ws = slot_base + p.ruw_doubles;
    double* vn = ws + (long long)VN * p.nmax;
    double* vext = ws + (long long)VEXT * p.nmax;
    double* vks = ws + (long long)VKS * p.nmax;
    double* nout = ws + (long long)VNOUT * p.nmax;
    double* vh = ws + (long long)VH * p.nmax;
    double* vxc = ws + (long long)VXC * p.nmax;
    double* kt = ws + (long long)VKT * p.nmax;
    double* X = ws + (long long)(VDIFF + slots) * p.nmax;
    double* Y = X + (long long)(p.kmax + 2) * p.nmax;  // after the forward scratch
    double* Bv = Y + (long long)p.kmax * p.nmax;
    double* gm = Bv + (long long)p.kmax * p.nmax;
    double* gv = gm + p.nmax;
    double* gn = gv + p.nmax;
    double* t1 = gn + p.nmax;
    double* t2 = t1 + p.nmax;
    // external potential
    {
      const int M = p.num_nuclei[b];
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) {
        double x = x0 + i * dx, v = 0.0;
        for (int m = 0; m < M; ++m) {
          double Rm = p.locations[(long long)b * p.max_nuclei + m];
          double Z = p.charges[(long long)b * p.max_nuclei + m];
          v -= Z * interaction_fn(p, x - Rm);
        }
        vext[i] = v;
        vn[i] = p.dens_in[off + i];
      }
      __syncwarp();
    }
    // forward quantities at n_t.  With reflection symmetry (jax_dft
    // kohn_sham_iteration) the XC functional sees s = P n with
    // P = (I + flip) / 2 and its outputs are flip-averaged; P is linear and
    // self-adjoint, so the reverse pass below applies P to the same places.
    const bool refl = p.reflect != 0;
    stage64(sm.s64a, vn, N, lane);
    hartree(p, N, dx, sm, vh, kt, lane);
    if (refl) {
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) sm.s64a[kPad64 + i] = 0.5 * (vn[i] + vn[N - 1 - i]);
      __syncwarp();
    }
    xc_eval(p, N, dx, sm, true, vxc, nullptr, refl, lane);
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) vks[i] = vh[i] + vxc[i] + vext[i];
    __syncwarp();
    EigStats est = {};
    int flags = eigen_solve<kBand, false>(p, N, dx, ne, K, vks, X, ruw, false, 0.0, sm, lane, est);
    double tee, gap;
    density_from_orbitals(p, N, dx, ne, K, X, nout, sm, tee, gap, lane);
    const double gE = p.a_genergy ? p.a_genergy[b] : 0.0;
    const double at = p.a_alpha;
    T* n32 = reinterpret_cast<T*>(sm.f32);
    T* u32 = n32 + (p.nmax + 2 * kPadMlp);
    T* gacc = u32 + (p.nmax + 2 * kPadMlp);
    T* rec = gacc + (p.nmax + 2 * kPadMlp);
    const T* W;
    T ninv;
    if constexpr (kNet64) {
      W = p.mlp_w64;
      ninv = p.mlp_norm_inv64;
    } else {
      W = sm.mlpw;
      ninv = p.mlp.norm_inv;
    }
    double acc[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) acc[q] = 0.0;
    // ---- gm, and the energy's explicit parameter dependence E_xc(m_t)
    if (gE != 0.0) {
      stage64(sm.s64a, nout, N, lane);
      hartree(p, N, dx, sm, t1, kt, lane);
      if (refl) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp)
          sm.s64a[kPad64 + i] = 0.5 * (nout[i] + nout[N - 1 - i]);
        __syncwarp();
      }
      xc_eval(p, N, dx, sm, true, t2, nullptr, refl, lane);
    }
    // the mixing reads the reflected output density: its cotangent is P gnext
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) {
      const double gx = refl ? 0.5 * (p.a_gnext[off + i] + p.a_gnext[off + N - 1 - i])
                             : p.a_gnext[off + i];
      double g = at * gx;
      if (gE != 0.0) g += gE * dx * (t1[i] + t2[i] + vext[i] - vks[i]);
      gm[i] = g;
    }
    __syncwarp();
    if (gE != 0.0) {
      // E_xc = dx sum eps_i(s) s_i at s = P m (s = m without reflection)
      const double* sm_out = nout;
      if (refl) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) t1[i] = 0.5 * (nout[i] + nout[N - 1 - i]);
        __syncwarp();
        sm_out = t1;
      }
      #pragma unroll 1
      for (int i = lane; i < N + 2 * kPadMlp; i += kWarp) {
        const int k = i - kPadMlp;
        n32[i] = (k >= 0 && k < N) ? (T)sm_out[k] * ninv : T(0);
        gacc[i] = T(0);
      }
      __syncwarp();
      // ybar_i = gE dx s_i (local convention E_xc = dx sum eps_i s_i); no tangent
      mlp_adjoint_pass(W, ninv, N, n32, n32, false, sm_out, gE * dx, sm_out, gacc, gn, rec, acc,
                       lane);
    }
    // ---- gv = chi gm
    sternheimer<kBand>(p, N, dx, ne, vks, X, gm, Y, Bv, gv, sm, lane);
    // ---- gn = (1 - a) gnext + v_H(gv) + d/dn[v_xc(n) . gv]
    stage64(sm.s64a, gv, N, lane);
    hartree(p, N, dx, sm, t1, kt, lane);
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) gn[i] = (1.0 - at) * p.a_gnext[off + i] + t1[i];
    {
      // with reflection: v_xc(n) . u = v(s) . (P u), s = P n, and the gradient
      // with respect to s goes back through P; vh and vxc are free here
      const double* sv = vn;
      const double* uv = gv;
      double* xg = gn;
      if (refl) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) {
          vh[i] = 0.5 * (vn[i] + vn[N - 1 - i]);
          vxc[i] = 0.5 * (gv[i] + gv[N - 1 - i]);
          t2[i] = 0.0;
        }
        __syncwarp();
        sv = vh;
        uv = vxc;
        xg = t2;
      }
      #pragma unroll 1
      for (int i = lane; i < N + 2 * kPadMlp; i += kWarp) {
        const int k = i - kPadMlp;
        n32[i] = (k >= 0 && k < N) ? (T)sv[k] * ninv : T(0);
        u32[i] = (k >= 0 && k < N) ? (T)uv[k] * ninv : T(0);
        gacc[i] = T(0);
      }
      __syncwarp();
      // local convention: v_xc(n) . u = sum_i [eps_i u_i + n_i D eps_i[u window]]
      mlp_adjoint_pass(W, ninv, N, n32, u32, true, uv, 1.0, sv, gacc, xg, rec, acc, lane);
      #pragma unroll 1
      for (int i = lane; i < N; i += kWarp) xg[i] += (double)gacc[i + kPadMlp];
      __syncwarp();
      if (refl) {
        #pragma unroll 1
        for (int i = lane; i < N; i += kWarp) gn[i] += 0.5 * (t2[i] + t2[N - 1 - i]);
        __syncwarp();
      }
    }
    #pragma unroll 1
    for (int i = lane; i < N; i += kWarp) p.a_gn[off + i] = gn[i];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const int pidx = lane + 32 * q;
      if (pidx < QEX_MLP_NUM_PARAMS) p.a_gtheta[(long long)b * QEX_MLP_NUM_PARAMS + pidx] += acc[q];
    }
    if (lane == 0 && p.o_status) p.o_status[b] = flags;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
thread_local int g_last_launches = 0;

int mix_slots_for(const qex_ks1d_options* o) {
  int m = o->num_mixing_iterations < 1 ? 1 : o->num_mixing_iterations;
  int it = o->num_iterations < 1 ? 1 : o->num_iterations;
  return m < it ? m : it;
}

int check_options(const qex_ks1d_options* o) {
  if (!o) return QEX_BAD_ARG;
  if (o->stencil != 3 && o->stencil != 5) return QEX_BAD_ARG;
  if (o->interaction != QEX_INTERACTION_EXPONENTIAL &&
      o->interaction != QEX_INTERACTION_SOFT_COULOMB)
    return QEX_BAD_ARG;
  if (o->num_iterations < 1 || o->max_num_grids < 5 || o->max_num_electrons < 1) return QEX_BAD_ARG;
  if (o->max_num_electrons / 2 + 1 > QEX_KS1D_MAX_EIGENPAIRS) return QEX_BAD_ARG;
  if (o->num_mixing_iterations < 1) return QEX_BAD_ARG;
  if (o->solve_planes < 0 || o->solve_planes > 2) return QEX_BAD_ARG;
  if (o->solve_chunk != 0 && o->solve_chunk != 16 && o->solve_chunk != 32 &&
      o->solve_chunk != kMaxChunk)
    return QEX_BAD_ARG;
  return QEX_OK;
}

long long stride_doubles(const qex_ks1d_options* o, bool adjoint = false) {
  int kmax = o->max_num_electrons / 2 + 1;
  long long v = vec_count(mix_slots_for(o), kmax);
  if (adjoint) v += 2LL * kmax + 5;  // Sternheimer solutions and right-hand sides, 5 vectors
  long long s = ruw_doubles(o->max_num_grids, kmax) + v * (long long)o->max_num_grids;
  return (s + 31) / 32 * 32;
}

// Bytes of the dense networks' scratch vectors (4 per slot) for a batch shape.
size_t nn_tail_bytes(const qex_ks1d_options* o, int num_molecules) {
  return sizeof(double) * 4 * (size_t)num_molecules * (size_t)o->max_num_grids;
}

// Bytes of the deferred KSR energy rows for a batch shape.
size_t ksr_defer_bytes(const qex_ks1d_options* o, int num_molecules) {
  return sizeof(double) * (size_t)num_molecules * (size_t)o->num_iterations *
         (size_t)o->max_num_grids;
}

int fill_params(Params& P, int mode, const qex_ks1d_batch* b, const qex_ks1d_options* o,
                const qex_xc_spec* xc, const qex_ks1d_outputs* out, void* ws, size_t ws_bytes,
                int num_molecules) {
  memset(&P, 0, sizeof(P));
  int rc = check_options(o);
  if (rc) return rc;
  if (!b || !xc) return QEX_BAD_ARG;
  P.mode = mode;
  P.num_molecules = num_molecules;
  P.order = b->order;
  P.num_grids = b->num_grids;
  P.grid_offsets = b->grid_offsets;
  P.grid_start = b->grid_start;
  P.grid_spacing = b->grid_spacing;
  P.num_electrons = b->num_electrons;
  P.num_nuclei = b->num_nuclei;
  P.locations = b->locations;
  P.charges = b->nuclear_charges;
  P.vext_in = b->external_potential;
  P.dens_in = b->initial_density;
  P.max_nuclei = o->max_nuclei;
  P.stencil = o->stencil;
  P.interaction = o->interaction;
  P.ia = o->interaction_a;
  P.ib = o->interaction_b;
  P.iters = o->num_iterations;
  P.alpha = o->alpha;
  P.alpha_decay = o->alpha_decay;
  P.mixing = o->num_mixing_iterations;
  P.tol = o->density_mse_converge_tolerance;
  P.rule = o->convergence_rule;
  P.reflect = o->enforce_reflection_symmetry;
  P.vext_given = o->external_potential_given;
  P.nmax = o->max_num_grids;
  P.kmax = o->max_num_electrons / 2 + 1;
  P.mix_slots = mix_slots_for(o);
  P.xc_kind = xc->kind;
  P.xc_conv = xc->convention;
  P.xc_a = xc->coefficient;
  P.xc_p = xc->power;
  P.xc_shift = xc->shift;
  P.lda_A = xc->lda_amplitude;
  P.lda_kappa = xc->lda_kappa;
  if (xc->kind < QEX_XC_NONE || xc->kind > QEX_XC_GLOBAL_MLP) return QEX_BAD_ARG;
  if (xc->convention != QEX_XC_AMPLITUDE && xc->convention != QEX_XC_LOCAL) return QEX_BAD_ARG;
  if (xc->kind == QEX_XC_WINDOW_MLP) {
    if (!fill_mlp_params(P.mlp, xc)) return QEX_BAD_ARG;
    if (xc->mlp_params64) {
      if (reinterpret_cast<uintptr_t>(xc->mlp_params64) % 16 != 0) return QEX_BAD_ARG;
      P.mlp_w64 = xc->mlp_params64;
      P.mlp_norm_inv64 = 1.0 / xc->normalization;
      // the FP64 windows, accumulator and per-lane scratch in the FP32 area
      P.nn_floats = 2 * (2 * (o->max_num_grids + 2 * kPadMlp) + kMlpScratch * kWarp);
    }
  }
  if (is_nn_kind(xc->kind)) {
    rc = fill_nn(P.nn, xc);
    if (rc) return rc;
    if (xc->kind == QEX_XC_GLOBAL_MLP && xc->nn_inputs > o->max_num_grids) return QEX_BAD_ARG;
    P.nn_floats = (int)nn_smem_floats(xc->kind, xc->nn_width, xc->nn_layers, o->max_num_grids);
  }
  if (xc->kind == QEX_XC_KSR) {
    if (!xc->ksr_params || reinterpret_cast<uintptr_t>(xc->ksr_params) % 16 != 0) return QEX_BAD_ARG;
    if (!(xc->ksr_maxval >= xc->ksr_minval) || !(xc->ksr_minval > 0.0)) return QEX_BAD_ARG;
    if (xc->ksr_channels != 8 && xc->ksr_channels != 16) return QEX_BAD_ARG;
    P.ksr_c = xc->ksr_channels;
    P.ksr_w = xc->ksr_params;
    P.ksr_lo = xc->ksr_minval;
    P.ksr_hi = xc->ksr_maxval;
  }
  if (out) {
    P.o_energy = out->total_energy;
    P.o_gap = out->gap;
    P.o_conv = out->converged;
    P.o_dens = out->density;
    P.o_vh = out->hartree_potential;
    P.o_vxc = out->xc_potential;
    P.o_f = out->xc_energy_density;
    P.o_final = out->final_density;
    P.o_vext = out->external_potential_out;
    P.o_status = out->status;
    P.o_iters = out->iterations_run;
    P.o_stats = out->stats;
    P.o_cycles = reinterpret_cast<long long*>(out->phase_cycles);
  }
  size_t need = 0;
  qex_ks1d_workspace_size(o, num_molecules, &need);
  if (!ws || ws_bytes < need) return QEX_BAD_ARG;
  if (reinterpret_cast<uintptr_t>(ws) % 16 != 0) return QEX_BAD_ARG;  // float4 solve area
  // KSR with a workspace of qex_ks1d_workspace_size_xc bytes: the energies'
  // E_xc on the output densities in one batched launch after the SCF
  if (mode == kModeScf && xc->kind == QEX_XC_KSR && out && out->total_energy) {
    const size_t base = (need + 255) / 256 * 256;
    if (ws_bytes >= base + ksr_defer_bytes(o, num_molecules))
      P.ksr_defer = reinterpret_cast<double*>(static_cast<unsigned char*>(ws) + base);
  }
  // dense networks: their scratch vectors follow the base workspace
  // (qex_ks1d_workspace_size_xc bytes in all)
  if (is_nn_kind(xc->kind)) {
    const size_t base = (need + 255) / 256 * 256;
    if (ws_bytes < base + nn_tail_bytes(o, num_molecules)) return QEX_BAD_ARG;
    P.nn_ws = reinterpret_cast<double*>(static_cast<unsigned char*>(ws) + base);
  }
  P.counter = reinterpret_cast<int*>(ws);
  P.ws = reinterpret_cast<double*>(static_cast<unsigned char*>(ws) + 256);
  P.stride = stride_doubles(o);
  P.ruw_doubles = ruw_doubles(o->max_num_grids, o->max_num_electrons / 2 + 1);
  P.planes = o->solve_planes;
  P.chunk = o->solve_chunk ? o->solve_chunk : kChunk;
  if (num_molecules < 0) return QEX_BAD_ARG;
  if (num_molecules > 0) {
    if (!b->num_grids || !b->grid_offsets || !b->grid_start || !b->grid_spacing ||
        !b->num_electrons)
      return QEX_BAD_ARG;
    if (!o->external_potential_given &&
        (!b->num_nuclei || !b->locations || !b->nuclear_charges || o->max_nuclei < 1))
      return QEX_BAD_ARG;
    if (o->external_potential_given && !b->external_potential) return QEX_BAD_ARG;
  }
  return QEX_OK;
}

// E_xc of the KSR network on the output densities the SCF kernel recorded in
// p.ksr_defer (rows (slot, iteration)), added to the recorded total energies.
// One warp per row with four channels' scans staged at a time: the SCF
// kernel's register cap allows one.  The network arithmetic per channel is
// the same as inside the SCF kernel.
template <int C>
__global__ void __launch_bounds__(kWarp) ksr_energy_kernel(const __grid_constant__ Params p) {
  extern __shared__ __align__(16) float ksm[];
  const int lane = threadIdx.x;
  const long long rows = (long long)p.num_molecules * p.iters;
  const bool local = (p.xc_conv == QEX_XC_LOCAL);
  for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int slot = (int)(row / p.iters), t = (int)(row % p.iters);
    const int b = p.order ? p.order[slot] : slot;
    const int N = p.num_grids[b];
    const int ne = p.num_electrons[b];
    const double dx = p.grid_spacing[b];
    if (N < 5 || N > p.nmax || ne < 1 || ne / 2 + 1 > p.kmax || !(dx > 0.0)) continue;
    const double e = ksr_eval<C, false, 4>(p.ksr_w, p.ksr_slot, p.ksr_lo, p.ksr_hi, N, dx,
                                           p.ksr_defer + row * p.nmax, local, nullptr, nullptr,
                                           ksm, lane);
    const double exc = warp_sum(e) * dx;
    if (lane == 0) p.o_energy[(long long)b * p.iters + t] += exc;
  }
}

template <int kBand, bool kNet64>
int launch_adjoint_variant(const Params& P, cudaStream_t stream, size_t smem, int sms) {
  auto fn = ks1d_adjoint_kernel<kBand, kNet64>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return QEX_CUDA_ERROR;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kWarp, smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)sms * per_sm;
  if (grid > P.num_molecules) grid = P.num_molecules;
  if (cudaMemsetAsync(P.counter, 0, sizeof(int), stream) != cudaSuccess) return QEX_CUDA_ERROR;
  fn<<<(unsigned)grid, kWarp, smem, stream>>>(P);
  if (cudaGetLastError() != cudaSuccess) return QEX_CUDA_ERROR;
  g_last_launches = 1;
  return QEX_OK;
}

int launch_adjoint(const Params& P, cudaStream_t stream) {
  g_last_launches = 0;
  if (P.num_molecules == 0) return QEX_OK;
  const SmemLayout L = smem_layout(P.nmax, P.kmax, true, false, P.nn_floats, P.chunk);
  const size_t smem = L.total;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
  int sms = 0, max_optin = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if ((int)smem > max_optin) return QEX_BAD_ARG;
  const bool net64 = P.mlp_w64 != nullptr;
  if (P.stencil == 5)
    return net64 ? launch_adjoint_variant<2, true>(P, stream, smem, sms)
                 : launch_adjoint_variant<2, false>(P, stream, smem, sms);
  return net64 ? launch_adjoint_variant<1, true>(P, stream, smem, sms)
               : launch_adjoint_variant<1, false>(P, stream, smem, sms);
}

template <int kBand, bool kRes, bool kKsr>
int launch_variant(const Params& P, cudaStream_t stream, size_t smem, int per_sm, int sms) {
  cudaError_t e = cudaFuncSetAttribute(ks1d_kernel<kBand, kRes, kKsr>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return QEX_CUDA_ERROR;
  long long grid = (long long)sms * per_sm;
  if (grid > P.num_molecules) grid = P.num_molecules;
  e = cudaMemsetAsync(P.counter, 0, sizeof(int), stream);
  if (e != cudaSuccess) return QEX_CUDA_ERROR;
  if constexpr (kKsr) {
    auto stage = ksr_stage(P.ksr_w, 6 * P.ksr_c * P.ksr_c + 2 * P.ksr_c, stream);
    if (stage.capturing_refused()) return QEX_BAD_ARG;
    if (stage.slot() < 0) return QEX_CUDA_ERROR;
    Params Q = P;
    Q.ksr_slot = stage.slot();
    ks1d_kernel<kBand, kRes, kKsr><<<(unsigned)grid, kWarp, smem, stream>>>(Q);
    bool ok = cudaGetLastError() == cudaSuccess;
    if (ok && Q.ksr_defer) {
      const size_t ks = sizeof(float) * ksr_scratch_floats(Q.nmax);
      auto fn = Q.ksr_c == 16 ? ksr_energy_kernel<16> : ksr_energy_kernel<8>;
      ok = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ks) ==
           cudaSuccess;
      long long rows = (long long)Q.num_molecules * Q.iters;
      if (rows > (1LL << 22)) rows = 1LL << 22;
      if (ok && rows > 0) {
        fn<<<(unsigned)rows, kWarp, ks, stream>>>(Q);
        ok = cudaGetLastError() == cudaSuccess;
      }
    }
    if (!stage.finish() || !ok) return QEX_CUDA_ERROR;
    g_last_launches = Q.ksr_defer ? 2 : 1;
    return QEX_OK;
  } else {
    ks1d_kernel<kBand, kRes, kKsr><<<(unsigned)grid, kWarp, smem, stream>>>(P);
    if (cudaGetLastError() != cudaSuccess) return QEX_CUDA_ERROR;
  }
  g_last_launches = 1;
  return QEX_OK;
}

template <int kBand, bool kRes, bool kKsr>
int blocks_per_sm(size_t smem) {
  int per_sm = 0;
  if (cudaFuncSetAttribute(ks1d_kernel<kBand, kRes, kKsr>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks1d_kernel<kBand, kRes, kKsr>, kWarp,
                                                smem);
  return per_sm;
}

// Picks the solve-plane placement: resident in shared memory when the whole
// batch fits in one wave of resident warps (lowest latency), streamed through
// the ring otherwise (a small shared-memory footprint, so more warps per SM).
int launch(const Params& P, cudaStream_t stream) {
  g_last_launches = 0;
  if (P.num_molecules == 0) return QEX_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
  int sms = 0, max_optin = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t smem_s = smem_layout(P.nmax, P.kmax, false, false, P.nn_floats, P.chunk).total;
  const size_t smem_r = smem_layout(P.nmax, P.kmax, false, true, P.nn_floats, P.chunk).total;
  const bool band2 = (P.stencil == 5);
  if (P.xc_kind == QEX_XC_KSR) {
    // the KSR instantiation streams its solve planes (one variant per stencil)
    if ((int)smem_s > max_optin) return QEX_BAD_ARG;
    int per = band2 ? blocks_per_sm<2, false, true>(smem_s) : blocks_per_sm<1, false, true>(smem_s);
    if (per < 1) per = 1;
    return band2 ? launch_variant<2, false, true>(P, stream, smem_s, per, sms)
                 : launch_variant<1, false, true>(P, stream, smem_s, per, sms);
  }
  if (P.planes != 2 && (int)smem_r <= max_optin) {
    const int per_r =
        band2 ? blocks_per_sm<2, true, false>(smem_r) : blocks_per_sm<1, true, false>(smem_r);
    if (per_r >= 1 && (P.planes == 1 || (long long)P.num_molecules <= (long long)sms * per_r)) {
      return band2 ? launch_variant<2, true, false>(P, stream, smem_r, per_r, sms)
                   : launch_variant<1, true, false>(P, stream, smem_r, per_r, sms);
    }
  }
  if (P.planes == 1 || (int)smem_s > max_optin) return QEX_BAD_ARG;
  int per_s =
      band2 ? blocks_per_sm<2, false, false>(smem_s) : blocks_per_sm<1, false, false>(smem_s);
  if (per_s < 1) per_s = 1;
  return band2 ? launch_variant<2, false, false>(P, stream, smem_s, per_s, sms)
               : launch_variant<1, false, false>(P, stream, smem_s, per_s, sms);
}

}  // namespace
}  // namespace qex

// Scratch of qex_ks1d_solve_static: a fixed device array, so that callers
// that cannot allocate device memory can still run the batched solver.  Every
// GPU that loads this library holds these 16 MiB until the process exits.
static constexpr size_t kStaticScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char qex_static_scratch[kStaticScratchBytes];

namespace {
constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mutex;
void* g_static_address[kStaticMaxDevices] = {};

// Device address of the scratch array on the current device.  Host code may
// not use the array's name as a pointer (it is a host-side stand-in), so the
// address is looked up with that device current.  Outside stream capture it
// is looked up on every call (cheap), so a device reset or a new primary
// context never leaves a stale address behind; under capture the address
// from the last call outside capture is used.
int static_scratch_address(cudaStream_t stream, void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QEX_CUDA_ERROR;
  if (dev < 0 || dev >= kStaticMaxDevices) return QEX_BAD_ARG;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) return QEX_CUDA_ERROR;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (cap == cudaStreamCaptureStatusNone || !g_static_address[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, qex_static_scratch) != cudaSuccess || !ptr) {
      return QEX_CUDA_ERROR;
    }
    g_static_address[dev] = ptr;
  }
  *out = g_static_address[dev];
  return QEX_OK;
}
}  // namespace

extern "C" {

int qex_ks1d_workspace_size(const qex_ks1d_options* options, int32_t num_molecules,
                            size_t* bytes) {
  if (!bytes) return QEX_BAD_ARG;
  *bytes = 0;
  int rc = qex::check_options(options);
  if (rc) return rc;
  if (num_molecules < 0) return QEX_BAD_ARG;
  *bytes = 256 + sizeof(double) * (size_t)qex::stride_doubles(options) * (size_t)num_molecules;
  return QEX_OK;
}

int qex_ks1d_workspace_size_xc(const qex_ks1d_options* options, const qex_xc_spec* xc,
                               int32_t num_molecules, size_t* bytes) {
  int rc = qex_ks1d_workspace_size(options, num_molecules, bytes);
  if (rc) return rc;
  if (xc && xc->kind == QEX_XC_KSR)
    *bytes = (*bytes + 255) / 256 * 256 + qex::ksr_defer_bytes(options, num_molecules);
  if (xc && qex::is_nn_kind(xc->kind))
    *bytes = (*bytes + 255) / 256 * 256 + qex::nn_tail_bytes(options, num_molecules);
  return QEX_OK;
}

int qex_ks1d_solve(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                   const qex_xc_spec* xc, const qex_ks1d_outputs* outputs, void* workspace,
                   size_t workspace_bytes, void* stream) {
  qex::Params P;
  if (!batch) return QEX_BAD_ARG;
  int rc = qex::fill_params(P, qex::kModeScf, batch, options, xc, outputs, workspace,
                            workspace_bytes, batch->num_molecules);
  if (rc) return rc;
  return qex::launch(P, static_cast<cudaStream_t>(stream));
}

int qex_ks1d_solve_static(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                          const qex_xc_spec* xc, const qex_ks1d_outputs* outputs, void* stream) {
  if (!batch) return QEX_BAD_ARG;
  size_t need = 0;
  int rc = qex_ks1d_workspace_size(options, batch->num_molecules, &need);
  if (rc) return rc;
  if (need > kStaticScratchBytes) return QEX_OOM;  // batch too large for the fixed scratch
  void* scratch = nullptr;
  rc = static_scratch_address(static_cast<cudaStream_t>(stream), &scratch);
  if (rc) return rc;
  qex::Params P;
  rc = qex::fill_params(P, qex::kModeScf, batch, options, xc, outputs, scratch,
                        kStaticScratchBytes, batch->num_molecules);
  if (rc) return rc;
  // the work counter at the start of the scratch is zeroed inside launch()
  return qex::launch(P, static_cast<cudaStream_t>(stream));
}

int qex_ks1d_iteration(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                       const qex_xc_spec* xc, const double* density_in,
                       const qex_ks1d_outputs* outputs, void* workspace, size_t workspace_bytes,
                       void* stream) {
  if (!batch || !density_in || !options) return QEX_BAD_ARG;
  qex_ks1d_options o = *options;
  o.num_iterations = 1;
  qex::Params P;
  int rc = qex::fill_params(P, qex::kModeIteration, batch, &o, xc, outputs, workspace,
                            workspace_bytes, batch->num_molecules);
  if (rc) return rc;
  P.dens_in = density_in;
  return qex::launch(P, static_cast<cudaStream_t>(stream));
}

int qex_ks1d_adjoint_workspace_size(const qex_ks1d_options* options, int32_t num_molecules,
                                    size_t* bytes) {
  if (!bytes) return QEX_BAD_ARG;
  *bytes = 0;
  int rc = qex::check_options(options);
  if (rc) return rc;
  if (num_molecules < 0) return QEX_BAD_ARG;
  *bytes = 256 + sizeof(double) * (size_t)qex::stride_doubles(options, true) * (size_t)num_molecules;
  return QEX_OK;
}

int qex_ks1d_adjoint_step(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                          const qex_xc_spec* xc, const double* density_in,
                          const double* grad_density_next, const double* grad_energy,
                          double alpha, double* grad_density, double* grad_params,
                          int32_t* status, void* workspace, size_t workspace_bytes,
                          void* stream) {
  if (!batch || !options || !xc || !density_in || !grad_density_next || !grad_density ||
      !grad_params)
    return QEX_BAD_ARG;
  if (xc->kind != QEX_XC_WINDOW_MLP || xc->convention != QEX_XC_LOCAL) return QEX_BAD_ARG;
  if (options->interaction != QEX_INTERACTION_EXPONENTIAL || options->external_potential_given ||
      options->num_mixing_iterations != 1)
    return QEX_BAD_ARG;
  size_t need = 0;
  int rc = qex_ks1d_adjoint_workspace_size(options, batch->num_molecules, &need);
  if (rc) return rc;
  if (!workspace || workspace_bytes < need) return QEX_BAD_ARG;
  qex_ks1d_options o = *options;
  o.num_iterations = 1;
  qex_ks1d_outputs out;
  memset(&out, 0, sizeof(out));
  out.status = status;
  qex::Params P;
  // fill_params checks the forward workspace size, which the adjoint one exceeds
  rc = qex::fill_params(P, qex::kModeIteration, batch, &o, xc, &out, workspace, workspace_bytes,
                        batch->num_molecules);
  if (rc) return rc;
  P.stride = qex::stride_doubles(&o, true);
  if (P.mlp_w64)  // FP64 windows and per-lane records of the adjoint's MLP passes
    P.nn_floats = 2 * (3 * (o.max_num_grids + 2 * qex::kPadMlp) + qex::kMlpRec * qex::kWarp);
  P.dens_in = density_in;
  P.a_gnext = grad_density_next;
  P.a_genergy = grad_energy;
  P.a_alpha = alpha;
  P.a_gn = grad_density;
  P.a_gtheta = grad_params;
  return qex::launch_adjoint(P, static_cast<cudaStream_t>(stream));
}

int qex_ks1d_noninteracting(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                            const double* potential, double* density, double* total_eigen_energy,
                            double* gap, int32_t* status, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (!batch || !potential || !options) return QEX_BAD_ARG;
  qex_ks1d_options o = *options;
  o.num_iterations = 1;
  o.external_potential_given = 1;
  qex_ks1d_batch bb = *batch;
  bb.external_potential = potential;
  qex_xc_spec xc;
  memset(&xc, 0, sizeof(xc));
  qex_ks1d_outputs out;
  memset(&out, 0, sizeof(out));
  out.final_density = density;
  out.status = status;
  qex::Params P;
  int rc = qex::fill_params(P, qex::kModeNonInteracting, &bb, &o, &xc, &out, workspace,
                            workspace_bytes, bb.num_molecules);
  if (rc) return rc;
  P.o_tee = total_eigen_energy;
  P.o_gap = gap;
  return qex::launch(P, static_cast<cudaStream_t>(stream));
}

const char* qex_version(void) { return "qex_gb300 0.1 (sm_103a)"; }

int qex_last_launch_count(void) { return qex::g_last_launches; }

}  // extern "C"
