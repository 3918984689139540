// Gaussian integrals over Cartesian s, p and d shells, McMurchie-Davidson
// (Helgaker, Joergensen, Olsen, "Molecular Electronic-Structure Theory",
// ch. 9): overlap, kinetic energy, nuclear attraction, and the three- and
// two-centre Coulomb integrals of density fitting, with the Cholesky factor of
// the fitting metric and the fitted factors B = L^-1 (Q|ij).  These replace
// pyscf's libcint (int1e_*_cart, int3c2e, int2c2e) as reached from the
// reference (qedft/train/td/hf.py:425-449 through pyscfad df_jk).
//
// One-electron: a warp per shell pair A <= B, its lanes over primitive pairs
// (overlap, kinetic) and over (primitive pair, nucleus) items (nuclear
// attraction), partials summed by a fixed shuffle tree and written to both
// triangles.  Three-centre: a thread per (A <= B, auxiliary shell); two-centre:
// a thread per auxiliary pair.  FP64 throughout.  The Boys function F_n(T),
// n <= 6, is a series times exp(-T) with downward recursion below T = 30 and
// erf with upward recursion above.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cart.cuh"
#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kL = kMaxShellL;
constexpr int kRMax = 3 * kL;                                         // (dd|d)
constexpr int kNC = ncart(kL);
constexpr double kPi = 3.141592653589793;

__device__ void boys(int nmax, double T, double* F) {
  if (T < 30.0) {
    // F_nmax = exp(-T) sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1))
    double term = 1.0 / (2 * nmax + 1), sum = term;
    for (int k = 0; k < 400; ++k) {
      term *= 2.0 * T / (2 * nmax + 2 * k + 3);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    const double e = exp(-T);
    F[nmax] = e * sum;
    for (int n = nmax; n > 0; --n) F[n - 1] = (2.0 * T * F[n] + e) / (2 * n - 1);
  } else {
    const double e = exp(-T);
    F[0] = 0.5 * sqrt(kPi / T) * erf(sqrt(T));
    for (int n = 0; n < nmax; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) / (2.0 * T);
  }
}

// E^{ij}_t for one direction, i <= kL, j <= JM, t <= i + j
template <int JM>
struct Herm {
  double e[kL + 1][JM + 1][kL + JM + 1];
};

template <int JM>
__device__ void hermite(double a, double b, double XAB, int imax, int jmax, Herm<JM>& H) {
  const double p = a + b;
  const double XPA = -b / p * XAB, XPB = a / p * XAB, h = 0.5 / p;
  for (int i = 0; i <= imax; ++i)
    for (int j = 0; j <= jmax; ++j)
      for (int t = 0; t <= kL + JM; ++t) H.e[i][j][t] = 0.0;
  H.e[0][0][0] = exp(-a * b / p * XAB * XAB);
  for (int j = 0; j < jmax; ++j)
    for (int t = 0; t <= j + 1; ++t)
      H.e[0][j + 1][t] = (t > 0 ? h * H.e[0][j][t - 1] : 0.0) + XPB * H.e[0][j][t] +
                         (t + 1 <= j ? (t + 1) * H.e[0][j][t + 1] : 0.0);
  for (int i = 0; i < imax; ++i)
    for (int j = 0; j <= jmax; ++j)
      for (int t = 0; t <= i + j + 1; ++t)
        H.e[i + 1][j][t] = (t > 0 ? h * H.e[i][j][t - 1] : 0.0) + XPA * H.e[i][j][t] +
                           (t + 1 <= i + j ? (t + 1) * H.e[i][j][t + 1] : 0.0);
}

// x^k exp(-g x^2) about its own centre as sum_t E_t d^t/dx^t exp(-g x^2), k <= 2
__device__ inline double self_e(int k, int t, double g) {
  if (k == 0) return 1.0;
  if (k == 1) return 0.5 / g;
  return t == 0 ? 0.5 / g : 0.25 / (g * g);
}

// packed index of R_tuv: levels s = t + u + v, then t, then u
__device__ inline int ridx(int t, int u, int v) {
  const int s = t + u + v;
  return s * (s + 1) * (s + 2) / 6 + t * (s + 1) - t * (t - 1) / 2 + u;
}

__host__ __device__ constexpr int num_r(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

template <int LM>
struct HermR {
  double r[num_r(LM)];
};

// R_tuv (t + u + v <= L <= LM) for exponent p and the vector (X, Y, Z)
template <int LM>
__device__ void hermite_r(int L, double p, double X, double Y, double Z, HermR<LM>& out) {
  double F[LM + 1], pw[LM + 1];
  boys(L, p * (X * X + Y * Y + Z * Z), F);
  pw[0] = 1.0;
  for (int n = 0; n < L; ++n) pw[n + 1] = pw[n] * (-2.0 * p);
  // R^n for n = L .. 0 in two buffers; the one holding n = 0 is out.r
  double tmp[num_r(LM)];
  double* cur = (L & 1) ? tmp : out.r;
  double* prv = (L & 1) ? out.r : tmp;
  cur[0] = pw[L] * F[L];
  for (int n = L - 1; n >= 0; --n) {
    double* t0 = cur;
    cur = prv;
    prv = t0;
    cur[0] = pw[n] * F[n];
    for (int s = 1; s <= L - n; ++s)
      for (int t = 0; t <= s; ++t)
        for (int u = 0; u <= s - t; ++u) {
          const int v = s - t - u;
          double val;
          if (t > 0)
            val = (t > 1 ? (t - 1) * prv[ridx(t - 2, u, v)] : 0.0) + X * prv[ridx(t - 1, u, v)];
          else if (u > 0)
            val = (u > 1 ? (u - 1) * prv[ridx(t, u - 2, v)] : 0.0) + Y * prv[ridx(t, u - 1, v)];
          else
            val = (v > 1 ? (v - 1) * prv[ridx(t, u, v - 2)] : 0.0) + Z * prv[ridx(t, u, v - 1)];
          cur[ridx(t, u, v)] = val;
        }
  }
}

// One-dimensional overlaps S_ij = int (x-A)^i (x-B)^j exp(-a(x-A)^2 - b(x-B)^2) dx,
// i <= kL, j <= kL + 2, by the Obara-Saika recurrence (J. Chem. Phys. 84,
// 3963 (1986)): S_{i+1,j} = X_PA S_ij + (i S_{i-1,j} + j S_{i,j-1}) / (2p), and
// the same with X_PB for j.
struct Ovl1 {
  double s[kL + 1][kL + 3];
};

__device__ void overlap_1d(double a, double b, double XAB, int imax, int jmax, Ovl1& O) {
  const double p = a + b;
  const double XPA = -b / p * XAB, XPB = a / p * XAB, h = 0.5 / p;
  O.s[0][0] = sqrt(kPi / p) * exp(-a * b / p * XAB * XAB);
  for (int j = 0; j < jmax; ++j)
    O.s[0][j + 1] = XPB * O.s[0][j] + (j > 0 ? h * j * O.s[0][j - 1] : 0.0);
  for (int i = 0; i < imax; ++i)
    for (int j = 0; j <= jmax; ++j)
      O.s[i + 1][j] = XPA * O.s[i][j] + h * ((i > 0 ? i * O.s[i - 1][j] : 0.0) +
                                             (j > 0 ? j * O.s[i][j - 1] : 0.0));
}

struct Shells {
  int ns;
  const double* centers;  // (ns, 3)
  const int* l;
  const int* poff;  // (ns + 1)
  const int* aoff;  // (ns)
  const double* ex;
  const double* co;
};

__device__ inline bool l_ok(int l) { return l >= 0 && l <= kL; }

// pair index -> (A, B >= A) over ns shells
__device__ inline void pair_of(long long pr, int ns, int& A, int& B) {
  A = 0;
  while (pr >= ns - A) {
    pr -= ns - A;
    ++A;
  }
  B = A + (int)pr;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// one-electron: S, T, V, a warp per shell pair A <= B
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) int1e_kernel(Shells sh, int n, int natom,
                                                         const double* __restrict__ Z,
                                                         const double* __restrict__ R,
                                                         double* S, double* T, double* V) {
  const int lane = threadIdx.x & 31;
  const long long npair = (long long)sh.ns * (sh.ns + 1) / 2;
  for (long long pr = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5); pr < npair;
       pr += (long long)gridDim.x * kWarps) {
    int A, B;
    pair_of(pr, sh.ns, A, B);
    const int la = sh.l[A], lb = sh.l[B];
    if (!l_ok(la) || !l_ok(lb)) continue;
    const int na = ncart(la), nb = ncart(lb);
    const int pa0 = sh.poff[A], npa = sh.poff[A + 1] - pa0;
    const int pb0 = sh.poff[B], npb = sh.poff[B + 1] - pb0;
    double AB[3], CA[3], CB[3];
    for (int d = 0; d < 3; ++d) {
      CA[d] = sh.centers[3 * A + d];
      CB[d] = sh.centers[3 * B + d];
      AB[d] = CA[d] - CB[d];
    }
    double s[kNC * kNC], kin[kNC * kNC], v[kNC * kNC];
    for (int q = 0; q < na * nb; ++q) s[q] = kin[q] = v[q] = 0.0;
    // overlap and kinetic energy: lanes over primitive pairs
    for (int it = lane; it < npa * npb; it += 32) {
      const int pa = pa0 + it / npb, pb = pb0 + it % npb;
      const double a = sh.ex[pa], b = sh.ex[pb], cc = sh.co[pa] * sh.co[pb];
      Ovl1 O[3];
      for (int d = 0; d < 3; ++d) overlap_1d(a, b, AB[d], la, lb + 2, O[d]);
      for (int ka = 0; ka < na; ++ka)
        for (int kb = 0; kb < nb; ++kb) {
          int ca[3], cb[3];
          cart_exponents(la, ka, ca);
          cart_exponents(lb, kb, cb);
          double s1[3], t1[3];
          for (int d = 0; d < 3; ++d) {
            // kinetic: -1/2 d^2/dx^2 on the ket, (x-B)^j -> j(j-1)(x-B)^(j-2)
            // - 2b(2j+1)(x-B)^j + 4b^2 (x-B)^(j+2)
            const int i = ca[d], j = cb[d];
            s1[d] = O[d].s[i][j];
            const double sm2 = j >= 2 ? O[d].s[i][j - 2] : 0.0;
            const double sp2 = O[d].s[i][j + 2];
            t1[d] = -0.5 * (j * (j - 1) * sm2 - 2.0 * b * (2 * j + 1) * s1[d] + 4.0 * b * b * sp2);
          }
          s[ka * nb + kb] += cc * s1[0] * s1[1] * s1[2];
          kin[ka * nb + kb] +=
              cc * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
        }
    }
    // nuclear attraction: lanes over (primitive pair, nucleus)
    for (int it = lane; it < npa * npb * natom; it += 32) {
      const int c = it % natom, pp = it / natom;
      const int pa = pa0 + pp / npb, pb = pb0 + pp % npb;
      const double a = sh.ex[pa], b = sh.ex[pb], p = a + b;
      const double pre = -sh.co[pa] * sh.co[pb] * Z[c] * 2.0 * kPi / p;
      Herm<kL> H[3];
      double PC[3];
      for (int d = 0; d < 3; ++d) {
        hermite(a, b, AB[d], la, lb, H[d]);
        PC[d] = (a * CA[d] + b * CB[d]) / p - R[3 * c + d];
      }
      HermR<2 * kL> Rr;
      hermite_r(la + lb, p, PC[0], PC[1], PC[2], Rr);
      for (int ka = 0; ka < na; ++ka)
        for (int kb = 0; kb < nb; ++kb) {
          int ca[3], cb[3];
          cart_exponents(la, ka, ca);
          cart_exponents(lb, kb, cb);
          double acc = 0.0;
          for (int t = 0; t <= ca[0] + cb[0]; ++t)
            for (int u = 0; u <= ca[1] + cb[1]; ++u)
              for (int w = 0; w <= ca[2] + cb[2]; ++w)
                acc += H[0].e[ca[0]][cb[0]][t] * H[1].e[ca[1]][cb[1]][u] *
                       H[2].e[ca[2]][cb[2]][w] * Rr.r[ridx(t, u, w)];
          v[ka * nb + kb] += pre * acc;
        }
    }
    for (int q = 0; q < na * nb; ++q) {
      const double sv = warp_sum(s[q]), tv = warp_sum(kin[q]), vv = warp_sum(v[q]);
      const int ka = q / nb, kb = q % nb;
      if (lane == 0 && (A != B || ka <= kb)) {
        const long long i = sh.aoff[A] + ka, j = sh.aoff[B] + kb;
        S[i * n + j] = S[j * n + i] = sv;
        T[i * n + j] = T[j * n + i] = tv;
        V[i * n + j] = V[j * n + i] = vv;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// (ij|P): one thread per (A <= B, C); writes both (i,j) and (j,i)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) int3c_kernel(Shells sh, Shells ax, int n,
                                                         double* __restrict__ out) {
  const long long npair = (long long)sh.ns * (sh.ns + 1) / 2;
  const long long total = npair * ax.ns;
  const double pi25 = 2.0 * pow(kPi, 2.5);
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int C = (int)(it % ax.ns);
    int A, B;
    pair_of(it / ax.ns, sh.ns, A, B);
    const int la = sh.l[A], lb = sh.l[B], lc = ax.l[C];
    if (!l_ok(la) || !l_ok(lb) || !l_ok(lc)) continue;
    const int na = ncart(la), nb = ncart(lb), nc = ncart(lc);
    double acc3[kNC * kNC * kNC];
    for (int q = 0; q < na * nb * nc; ++q) acc3[q] = 0.0;
    double AB[3];
    for (int d = 0; d < 3; ++d) AB[d] = sh.centers[3 * A + d] - sh.centers[3 * B + d];
    for (int pa = sh.poff[A]; pa < sh.poff[A + 1]; ++pa)
      for (int pb = sh.poff[B]; pb < sh.poff[B + 1]; ++pb) {
        const double a = sh.ex[pa], b = sh.ex[pb], p = a + b;
        Herm<kL> H[3];
        for (int d = 0; d < 3; ++d) hermite(a, b, AB[d], la, lb, H[d]);
        double P[3];
        for (int d = 0; d < 3; ++d) P[d] = (a * sh.centers[3 * A + d] + b * sh.centers[3 * B + d]) / p;
        for (int pc = ax.poff[C]; pc < ax.poff[C + 1]; ++pc) {
          const double g = ax.ex[pc];
          const double al = p * g / (p + g);
          const double pre = sh.co[pa] * sh.co[pb] * ax.co[pc] * pi25 / (p * g * sqrt(p + g));
          HermR<kRMax> Rr;
          hermite_r(la + lb + lc, al, P[0] - ax.centers[3 * C], P[1] - ax.centers[3 * C + 1],
                    P[2] - ax.centers[3 * C + 2], Rr);
          for (int ka = 0; ka < na; ++ka)
            for (int kb = 0; kb < nb; ++kb) {
              int ca[3], cb[3];
              cart_exponents(la, ka, ca);
              cart_exponents(lb, kb, cb);
              for (int kc = 0; kc < nc; ++kc) {
                int cc[3];
                cart_exponents(lc, kc, cc);
                double acc = 0.0;
                for (int t = 0; t <= ca[0] + cb[0]; ++t)
                  for (int u = 0; u <= ca[1] + cb[1]; ++u)
                    for (int w = 0; w <= ca[2] + cb[2]; ++w) {
                      const double e1 = H[0].e[ca[0]][cb[0]][t] * H[1].e[ca[1]][cb[1]][u] *
                                        H[2].e[ca[2]][cb[2]][w];
                      // the auxiliary Gaussian about its own centre, ket sign (-1)^(tt+uu+vv)
                      for (int tt = cc[0] & 1; tt <= cc[0]; tt += 2)
                        for (int uu = cc[1] & 1; uu <= cc[1]; uu += 2)
                          for (int vv = cc[2] & 1; vv <= cc[2]; vv += 2) {
                            const double ec = self_e(cc[0], tt, g) * self_e(cc[1], uu, g) *
                                              self_e(cc[2], vv, g);
                            const double sg = ((tt + uu + vv) & 1) ? -1.0 : 1.0;
                            acc += e1 * sg * ec * Rr.r[ridx(t + tt, u + uu, w + vv)];
                          }
                    }
                acc3[(kc * na + ka) * nb + kb] += pre * acc;
              }
            }
        }
      }
    const long long nn = (long long)n * n;
    for (int kc = 0; kc < nc; ++kc)
      for (int ka = 0; ka < na; ++ka)
        for (int kb = 0; kb < nb; ++kb) {
          if (A == B && kb < ka) continue;  // the mirror of (kb, ka) covers it
          const long long q = (long long)(ax.aoff[C] + kc) * nn;
          const int i = sh.aoff[A] + ka, j = sh.aoff[B] + kb;
          const double val = acc3[(kc * na + ka) * nb + kb];
          out[q + (long long)i * n + j] = val;
          out[q + (long long)j * n + i] = val;
        }
  }
}

// (P|Q): one thread per auxiliary shell pair
__global__ void __launch_bounds__(kThreads) int2c_kernel(Shells ax, int na,
                                                         double* __restrict__ out) {
  const long long total = (long long)ax.ns * ax.ns;
  const double pi25 = 2.0 * pow(kPi, 2.5);
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int A = (int)(it / ax.ns), B = (int)(it % ax.ns);
    const int la = ax.l[A], lb = ax.l[B];
    if (!l_ok(la) || !l_ok(lb)) continue;
    const int nA = ncart(la), nB = ncart(lb);
    double acc2[kNC * kNC];
    for (int q = 0; q < nA * nB; ++q) acc2[q] = 0.0;
    for (int pa = ax.poff[A]; pa < ax.poff[A + 1]; ++pa)
      for (int pb = ax.poff[B]; pb < ax.poff[B + 1]; ++pb) {
        const double a = ax.ex[pa], b = ax.ex[pb];
        const double al = a * b / (a + b);
        const double pre = ax.co[pa] * ax.co[pb] * pi25 / (a * b * sqrt(a + b));
        HermR<2 * kL> Rr;
        hermite_r(la + lb, al, ax.centers[3 * A] - ax.centers[3 * B],
                  ax.centers[3 * A + 1] - ax.centers[3 * B + 1],
                  ax.centers[3 * A + 2] - ax.centers[3 * B + 2], Rr);
        for (int ka = 0; ka < nA; ++ka)
          for (int kb = 0; kb < nB; ++kb) {
            int ca[3], cb[3];
            cart_exponents(la, ka, ca);
            cart_exponents(lb, kb, cb);
            double acc = 0.0;
            for (int t = ca[0] & 1; t <= ca[0]; t += 2)
              for (int u = ca[1] & 1; u <= ca[1]; u += 2)
                for (int w = ca[2] & 1; w <= ca[2]; w += 2) {
                  const double ea = self_e(ca[0], t, a) * self_e(ca[1], u, a) * self_e(ca[2], w, a);
                  for (int tt = cb[0] & 1; tt <= cb[0]; tt += 2)
                    for (int uu = cb[1] & 1; uu <= cb[1]; uu += 2)
                      for (int vv = cb[2] & 1; vv <= cb[2]; vv += 2) {
                        const double eb =
                            self_e(cb[0], tt, b) * self_e(cb[1], uu, b) * self_e(cb[2], vv, b);
                        const double sg = ((tt + uu + vv) & 1) ? -1.0 : 1.0;
                        acc += ea * eb * sg * Rr.r[ridx(t + tt, u + uu, w + vv)];
                      }
                }
            acc2[ka * nB + kb] += pre * acc;
          }
      }
    for (int ka = 0; ka < nA; ++ka)
      for (int kb = 0; kb < nB; ++kb)
        out[(long long)(ax.aoff[A] + ka) * na + ax.aoff[B] + kb] = acc2[ka * nB + kb];
  }
}

// ---------------------------------------------------------------------------
// Cholesky of the metric (lower, in place, one CTA) and B = L^-1 Y
// ---------------------------------------------------------------------------
constexpr int kCholThreads = 1024;

__global__ void __launch_bounds__(kCholThreads) chol_kernel(int m, double* __restrict__ A,
                                                            int* __restrict__ status) {
  __shared__ double piv;
  for (int k = 0; k < m; ++k) {
    if (threadIdx.x == 0) {
      const double d = A[(long long)k * m + k];
      piv = d > 0.0 ? sqrt(d) : 0.0;
      if (!(d > 0.0)) *status = QEX_NUMERICAL;
      A[(long long)k * m + k] = piv;
    }
    __syncthreads();
    if (piv == 0.0) return;
    for (int i = k + 1 + threadIdx.x; i < m; i += kCholThreads) A[(long long)i * m + k] /= piv;
    __syncthreads();
    const long long rest = (long long)(m - k - 1) * (m - k - 1);
    for (long long e = threadIdx.x; e < rest; e += kCholThreads) {
      const int i = k + 1 + (int)(e / (m - k - 1)), j = k + 1 + (int)(e % (m - k - 1));
      if (j <= i) A[(long long)i * m + j] -= A[(long long)i * m + k] * A[(long long)j * m + k];
    }
    __syncthreads();
  }
}

// forward substitution, one thread per column of Y (m x cols, row-major)
__global__ void __launch_bounds__(kThreads) trsm_kernel(int m, long long cols,
                                                        const double* __restrict__ L,
                                                        double* __restrict__ Y) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cols;
       c += (long long)gridDim.x * blockDim.x) {
    for (int i = 0; i < m; ++i) {
      double s = Y[(long long)i * cols + c];
      for (int k = 0; k < i; ++k) s -= L[(long long)i * m + k] * Y[(long long)k * cols + c];
      Y[(long long)i * cols + c] = s / L[(long long)i * m + i];
    }
  }
}

int grid_for(long long work) {
  long long g = (work + kThreads - 1) / kThreads;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

Shells make(int32_t ns, const double* c, const int32_t* l, const int32_t* poff, const int32_t* aoff,
            const double* ex, const double* co) {
  return Shells{ns, c, l, poff, aoff, ex, co};
}

}  // namespace

extern "C" {

int qex_td_int1e(int32_t num_shells, const double* centers, const int32_t* l,
                 const int32_t* prim_offset, const int32_t* ao_offset, const double* exponents,
                 const double* coefficients, int32_t nao, int32_t natom, const double* charges,
                 const double* positions, double* S, double* T, double* V, void* stream) {
  if (num_shells < 1 || nao < 1 || natom < 0) return QEX_BAD_ARG;
  if (!centers || !l || !prim_offset || !ao_offset || !exponents || !coefficients || !S || !T ||
      !V || (natom > 0 && (!charges || !positions)))
    return QEX_BAD_ARG;
  Shells sh = make(num_shells, centers, l, prim_offset, ao_offset, exponents, coefficients);
  const long long npair = (long long)num_shells * (num_shells + 1) / 2;
  int1e_kernel<<<grid_for(npair * 32), kThreads, 0,
                 static_cast<cudaStream_t>(stream)>>>(sh, nao, natom, charges, positions, S, T, V);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_int3c2e(int32_t num_shells, const double* centers, const int32_t* l,
                   const int32_t* prim_offset, const int32_t* ao_offset, const double* exponents,
                   const double* coefficients, int32_t nao, int32_t num_aux_shells,
                   const double* aux_centers, const int32_t* aux_l, const int32_t* aux_prim_offset,
                   const int32_t* aux_offset, const double* aux_exponents,
                   const double* aux_coefficients, int32_t naux, double* out, void* stream) {
  if (num_shells < 1 || nao < 1 || num_aux_shells < 1 || naux < 1 || !out) return QEX_BAD_ARG;
  if (!centers || !l || !prim_offset || !ao_offset || !exponents || !coefficients ||
      !aux_centers || !aux_l || !aux_prim_offset || !aux_offset || !aux_exponents ||
      !aux_coefficients)
    return QEX_BAD_ARG;
  Shells sh = make(num_shells, centers, l, prim_offset, ao_offset, exponents, coefficients);
  Shells ax = make(num_aux_shells, aux_centers, aux_l, aux_prim_offset, aux_offset, aux_exponents,
                   aux_coefficients);
  const long long work = (long long)num_shells * (num_shells + 1) / 2 * num_aux_shells;
  int3c_kernel<<<grid_for(work), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(sh, ax, nao,
                                                                                  out);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_int2c2e(int32_t num_aux_shells, const double* aux_centers, const int32_t* aux_l,
                   const int32_t* aux_prim_offset, const int32_t* aux_offset,
                   const double* aux_exponents, const double* aux_coefficients, int32_t naux,
                   double* out, void* stream) {
  if (num_aux_shells < 1 || naux < 1 || !out || !aux_centers || !aux_l || !aux_prim_offset ||
      !aux_offset || !aux_exponents || !aux_coefficients)
    return QEX_BAD_ARG;
  Shells ax = make(num_aux_shells, aux_centers, aux_l, aux_prim_offset, aux_offset, aux_exponents,
                   aux_coefficients);
  int2c_kernel<<<grid_for((long long)num_aux_shells * num_aux_shells), kThreads, 0,
                 static_cast<cudaStream_t>(stream)>>>(ax, naux, out);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

int qex_td_df_factors(int32_t naux, int64_t cols, double* metric, double* int3c,
                      int32_t* status, void* stream) {
  if (naux < 1 || cols < 1 || !metric || !int3c || !status) return QEX_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(status, 0, sizeof(int32_t), s) != cudaSuccess) return QEX_CUDA_ERROR;
  chol_kernel<<<1, kCholThreads, 0, s>>>(naux, metric, status);
  trsm_kernel<<<grid_for(cols), kThreads, 0, s>>>(naux, cols, metric, int3c);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}

}  // extern "C"
