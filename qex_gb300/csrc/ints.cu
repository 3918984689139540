// Gaussian integrals over Cartesian s and p shells, McMurchie-Davidson
// (Helgaker, Joergensen, Olsen, "Molecular Electronic-Structure Theory",
// ch. 9): overlap, kinetic energy, nuclear attraction, and the three- and
// two-centre Coulomb integrals of density fitting, with the Cholesky factor of
// the fitting metric and the fitted factors B = L^-1 (Q|ij).  These replace
// pyscf's libcint (int1e_*, int3c2e, int2c2e) as reached from the reference
// (qedft/train/td/hf.py:425-449 through pyscfad df_jk).
//
// One thread per shell pair (one-electron), shell triple (three-centre) or
// auxiliary pair (two-centre), looping over primitives; FP64 throughout.
// The Boys function F_n(T), n <= 4, is a series times exp(-T) with downward
// recursion below T = 30 and erf with upward recursion above.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kThreads = 128;
constexpr int kMaxL = 4;  // highest Boys order / Hermite rank needed (l <= 1 per centre, +1 slack)

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
    F[0] = 0.5 * sqrt(3.141592653589793 / T) * erf(sqrt(T));
    for (int n = 0; n < nmax; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) / (2.0 * T);
  }
}

// E^{ij}_t for one direction, i <= 1, j <= 3 (kinetic needs j + 2), t <= i + j
struct Herm {
  double e[2][4][5];
};

__device__ void hermite(double a, double b, double XAB, int imax, int jmax, Herm& H) {
  const double p = a + b;
  const double XPA = -b / p * XAB, XPB = a / p * XAB, h = 0.5 / p;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 4; ++j)
      for (int t = 0; t < 5; ++t) H.e[i][j][t] = 0.0;
  H.e[0][0][0] = exp(-a * b / p * XAB * XAB);
  for (int j = 0; j < jmax; ++j)
    for (int t = 0; t <= j + 1; ++t)
      H.e[0][j + 1][t] = (t > 0 ? h * H.e[0][j][t - 1] : 0.0) + XPB * H.e[0][j][t] +
                         (t + 1 <= j ? (t + 1) * H.e[0][j][t + 1] : 0.0);
  if (imax > 0)
    for (int j = 0; j <= jmax; ++j)
      for (int t = 0; t <= j + 1; ++t)
        H.e[1][j][t] = (t > 0 ? h * H.e[0][j][t - 1] : 0.0) + XPA * H.e[0][j][t] +
                       (t + 1 <= j ? (t + 1) * H.e[0][j][t + 1] : 0.0);
}

// R_{tuv} for t + u + v <= L (flat index tuv over [0,L]^3)
struct HermR {
  double r[kMaxL][kMaxL][kMaxL];
};

__device__ void hermite_r(int L, double p, double X, double Y, double Z, HermR& out) {
  double F[kMaxL + 1];
  boys(L, p * (X * X + Y * Y + Z * Z), F);
  // R^n_{tuv} built for decreasing n: level n needs t+u+v <= L-n
  double cur[kMaxL][kMaxL][kMaxL], nxt[kMaxL][kMaxL][kMaxL];
  for (int t = 0; t < kMaxL; ++t)
    for (int u = 0; u < kMaxL; ++u)
      for (int v = 0; v < kMaxL; ++v) nxt[t][u][v] = 0.0;
  double pw = 1.0;
  for (int n = 0; n < L; ++n) pw *= -2.0 * p;
  for (int n = L; n >= 0; --n) {
    for (int t = 0; t < kMaxL; ++t)
      for (int u = 0; u < kMaxL; ++u)
        for (int v = 0; v < kMaxL; ++v) cur[t][u][v] = 0.0;
    cur[0][0][0] = pw * F[n];
    const int top = L - n;
    for (int s = 1; s <= top; ++s)
      for (int t = 0; t <= s; ++t)
        for (int u = 0; u <= s - t; ++u) {
          const int v = s - t - u;
          double val;
          if (t > 0)
            val = (t > 1 ? (t - 1) * nxt[t - 2][u][v] : 0.0) + X * nxt[t - 1][u][v];
          else if (u > 0)
            val = (u > 1 ? (u - 1) * nxt[t][u - 2][v] : 0.0) + Y * nxt[t][u - 1][v];
          else
            val = (v > 1 ? (v - 1) * nxt[t][u][v - 2] : 0.0) + Z * nxt[t][u][v - 1];
          cur[t][u][v] = val;
        }
    for (int t = 0; t < kMaxL; ++t)
      for (int u = 0; u < kMaxL; ++u)
        for (int v = 0; v < kMaxL; ++v) nxt[t][u][v] = cur[t][u][v];
    if (n > 0) pw /= -2.0 * p;
  }
  for (int t = 0; t < kMaxL; ++t)
    for (int u = 0; u < kMaxL; ++u)
      for (int v = 0; v < kMaxL; ++v) out.r[t][u][v] = nxt[t][u][v];
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

__device__ int ncart(int l) { return l == 0 ? 1 : 3; }
__device__ void cart(int l, int k, int* c) {
  c[0] = c[1] = c[2] = 0;
  if (l == 1) c[k] = 1;
}

// ---------------------------------------------------------------------------
// one-electron: S, T, V over all shell pairs
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) int1e_kernel(Shells sh, int n, int natom,
                                                         const double* __restrict__ Z,
                                                         const double* __restrict__ R,
                                                         double* S, double* T, double* V) {
  const long long total = (long long)sh.ns * sh.ns;
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int A = (int)(it / sh.ns), B = (int)(it % sh.ns);
    const int la = sh.l[A], lb = sh.l[B];
    double s[3][3] = {}, kin[3][3] = {}, v[3][3] = {};
    double AB[3];
    for (int d = 0; d < 3; ++d) AB[d] = sh.centers[3 * A + d] - sh.centers[3 * B + d];
    for (int pa = sh.poff[A]; pa < sh.poff[A + 1]; ++pa)
      for (int pb = sh.poff[B]; pb < sh.poff[B + 1]; ++pb) {
        const double a = sh.ex[pa], b = sh.ex[pb], p = a + b, cc = sh.co[pa] * sh.co[pb];
        Herm H[3];
        for (int d = 0; d < 3; ++d) hermite(a, b, AB[d], la, lb + 2, H[d]);
        const double sq = sqrt(3.141592653589793 / p);
        double P[3];
        for (int d = 0; d < 3; ++d) P[d] = (a * sh.centers[3 * A + d] + b * sh.centers[3 * B + d]) / p;
        for (int ka = 0; ka < ncart(la); ++ka)
          for (int kb = 0; kb < ncart(lb); ++kb) {
            int ca[3], cb[3];
            cart(la, ka, ca);
            cart(lb, kb, cb);
            double s1[3], t1[3];
            for (int d = 0; d < 3; ++d) {
              const int i = ca[d], j = cb[d];
              s1[d] = H[d].e[i][j][0] * sq;
              const double sm2 = j >= 2 ? H[d].e[i][j - 2][0] * sq : 0.0;
              const double sp2 = H[d].e[i][j + 2][0] * sq;
              t1[d] = -0.5 * (j * (j - 1) * sm2 - 2.0 * b * (2 * j + 1) * s1[d] + 4.0 * b * b * sp2);
            }
            s[ka][kb] += cc * s1[0] * s1[1] * s1[2];
            kin[ka][kb] += cc * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
            const int L = la + lb;
            for (int c = 0; c < natom; ++c) {
              HermR Rr;
              hermite_r(L, p, P[0] - R[3 * c], P[1] - R[3 * c + 1], P[2] - R[3 * c + 2], Rr);
              double acc = 0.0;
              for (int t = 0; t <= ca[0] + cb[0]; ++t)
                for (int u = 0; u <= ca[1] + cb[1]; ++u)
                  for (int w = 0; w <= ca[2] + cb[2]; ++w)
                    acc += H[0].e[ca[0]][cb[0]][t] * H[1].e[ca[1]][cb[1]][u] *
                           H[2].e[ca[2]][cb[2]][w] * Rr.r[t][u][w];
              v[ka][kb] -= cc * Z[c] * 2.0 * 3.141592653589793 / p * acc;
            }
          }
      }
    for (int ka = 0; ka < ncart(la); ++ka)
      for (int kb = 0; kb < ncart(lb); ++kb) {
        const long long idx = (long long)(sh.aoff[A] + ka) * n + sh.aoff[B] + kb;
        S[idx] = s[ka][kb];
        T[idx] = kin[ka][kb];
        V[idx] = v[ka][kb];
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
  const double pi25 = 2.0 * pow(3.141592653589793, 2.5);
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int C = (int)(it % ax.ns);
    long long pr = it / ax.ns;
    int A = 0;
    while (pr >= sh.ns - A) {  // pair index -> (A, B >= A)
      pr -= sh.ns - A;
      ++A;
    }
    const int B = A + (int)pr;
    const int la = sh.l[A], lb = sh.l[B], lc = ax.l[C];
    double acc3[3][3][3] = {};
    double AB[3];
    for (int d = 0; d < 3; ++d) AB[d] = sh.centers[3 * A + d] - sh.centers[3 * B + d];
    for (int pa = sh.poff[A]; pa < sh.poff[A + 1]; ++pa)
      for (int pb = sh.poff[B]; pb < sh.poff[B + 1]; ++pb) {
        const double a = sh.ex[pa], b = sh.ex[pb], p = a + b;
        Herm H[3];
        for (int d = 0; d < 3; ++d) hermite(a, b, AB[d], la, lb, H[d]);
        double P[3];
        for (int d = 0; d < 3; ++d) P[d] = (a * sh.centers[3 * A + d] + b * sh.centers[3 * B + d]) / p;
        for (int pc = ax.poff[C]; pc < ax.poff[C + 1]; ++pc) {
          const double g = ax.ex[pc];
          const double al = p * g / (p + g);
          const double pre = sh.co[pa] * sh.co[pb] * ax.co[pc] * pi25 / (p * g * sqrt(p + g));
          HermR Rr;
          hermite_r(la + lb + lc, al, P[0] - ax.centers[3 * C], P[1] - ax.centers[3 * C + 1],
                    P[2] - ax.centers[3 * C + 2], Rr);
          for (int ka = 0; ka < ncart(la); ++ka)
            for (int kb = 0; kb < ncart(lb); ++kb) {
              int ca[3], cb[3];
              cart(la, ka, ca);
              cart(lb, kb, cb);
              for (int kc = 0; kc < ncart(lc); ++kc) {
                int cc[3];
                cart(lc, kc, cc);
                double acc = 0.0;
                for (int t = 0; t <= ca[0] + cb[0]; ++t)
                  for (int u = 0; u <= ca[1] + cb[1]; ++u)
                    for (int w = 0; w <= ca[2] + cb[2]; ++w) {
                      const double e1 = H[0].e[ca[0]][cb[0]][t] * H[1].e[ca[1]][cb[1]][u] *
                                        H[2].e[ca[2]][cb[2]][w];
                      // the auxiliary Gaussian about its own centre: x^1 -> E_1 = 1/(2g),
                      // with the ket sign (-1)^1
                      const int tt = cc[0], uu = cc[1], vv = cc[2];
                      const double ec = (tt + uu + vv) ? -0.5 / g : 1.0;
                      acc += e1 * ec * Rr.r[t + tt][u + uu][w + vv];
                    }
                acc3[kc][ka][kb] += pre * acc;
              }
            }
        }
      }
    const long long nn = (long long)n * n;
    for (int kc = 0; kc < ncart(lc); ++kc)
      for (int ka = 0; ka < ncart(la); ++ka)
        for (int kb = 0; kb < ncart(lb); ++kb) {
          const long long q = (long long)(ax.aoff[C] + kc) * nn;
          const int i = sh.aoff[A] + ka, j = sh.aoff[B] + kb;
          out[q + (long long)i * n + j] = acc3[kc][ka][kb];
          out[q + (long long)j * n + i] = acc3[kc][ka][kb];
        }
  }
}

// (P|Q): one thread per auxiliary shell pair
__global__ void __launch_bounds__(kThreads) int2c_kernel(Shells ax, int na,
                                                         double* __restrict__ out) {
  const long long total = (long long)ax.ns * ax.ns;
  const double pi25 = 2.0 * pow(3.141592653589793, 2.5);
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int A = (int)(it / ax.ns), B = (int)(it % ax.ns);
    const int la = ax.l[A], lb = ax.l[B];
    double acc2[3][3] = {};
    for (int pa = ax.poff[A]; pa < ax.poff[A + 1]; ++pa)
      for (int pb = ax.poff[B]; pb < ax.poff[B + 1]; ++pb) {
        const double a = ax.ex[pa], b = ax.ex[pb];
        const double al = a * b / (a + b);
        const double pre = ax.co[pa] * ax.co[pb] * pi25 / (a * b * sqrt(a + b));
        HermR Rr;
        hermite_r(la + lb, al, ax.centers[3 * A] - ax.centers[3 * B],
                  ax.centers[3 * A + 1] - ax.centers[3 * B + 1],
                  ax.centers[3 * A + 2] - ax.centers[3 * B + 2], Rr);
        for (int ka = 0; ka < ncart(la); ++ka)
          for (int kb = 0; kb < ncart(lb); ++kb) {
            int ca[3], cb[3];
            cart(la, ka, ca);
            cart(lb, kb, cb);
            const double ea = (ca[0] + ca[1] + ca[2]) ? 0.5 / a : 1.0;
            const double eb = (cb[0] + cb[1] + cb[2]) ? -0.5 / b : 1.0;
            acc2[ka][kb] += pre * ea * eb *
                            Rr.r[ca[0] + cb[0]][ca[1] + cb[1]][ca[2] + cb[2]];
          }
      }
    for (int ka = 0; ka < ncart(la); ++ka)
      for (int kb = 0; kb < ncart(lb); ++kb)
        out[(long long)(ax.aoff[A] + ka) * na + ax.aoff[B] + kb] = acc2[ka][kb];
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
  int1e_kernel<<<grid_for((long long)num_shells * num_shells), kThreads, 0,
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
