// Molecular integration grids: atom-centred radial x angular grids with
// Becke's fuzzy-cell partition (Becke, J. Chem. Phys. 88, 2547 (1988)), its
// atomic-size adjustment, and Stratmann's switching function (Stratmann,
// Scuseria, Frisch, Chem. Phys. Lett. 257, 213 (1996)): what
// pyscf.dft.gen_grid.Grids with becke_scheme = stratmann builds for the
// reference (qedft/data_io/td/dataset_generation.py:139-142,
// qedft/train/td/rks_legacy.py:46).
//
// One thread per grid point (atom a, radial node i, angular node j):
//   x = R_a + r_i u_j,  w = w_i w_j P_a(x) / sum_b P_b(x),
//   P_b(x) = prod_{c != b} s(nu_bc),  mu_bc = (|x - R_b| - |x - R_c|) / |R_b - R_c|,
//   nu_bc = mu_bc + a_bc (1 - mu_bc^2)   (size adjustment, a_bc precomputed),
//   s = (1 - g) / 2, g = Stratmann's polynomial in mu / 0.64 (Becke's
//   iterated polynomial with becke = 1).
// The radial and angular nodes come from the host (small tables); FP64.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "qex_ks1d.h"
#include "qex_td.h"

namespace {

constexpr int kThreads = 128;
constexpr int kMaxAtoms = 256;

__device__ double switch_s(double mu, int scheme) {
  double g;
  if (scheme == 1) {  // Stratmann, a = 0.64
    const double a = 0.64;
    if (mu <= -a) return 1.0;
    if (mu >= a) return 0.0;
    const double m = mu / a, m2 = m * m;
    g = (1.0 / 16.0) * m * (35.0 + m2 * (-35.0 + m2 * (21.0 - 5.0 * m2)));
  } else {  // Becke: three iterations of p(m) = 1.5 m - 0.5 m^3
    g = mu;
    for (int k = 0; k < 3; ++k) g = (3.0 - g * g) * g * 0.5;
  }
  return 0.5 * (1.0 - g);
}

struct GridParams {
  int natom;
  const double* xyz;      // (natom, 3)
  const double* adj;      // (natom, natom) size adjustment a_bc, or NULL
  const int64_t* off;     // (natom + 1) first point of each atom
  const int* nrad;        // (natom)
  const int64_t* roff;    // (natom) first radial node of each atom
  const double* rad_r;    // radial nodes (packed)
  const double* rad_w;    // radial weights, r^2 dr included (packed)
  int nang;
  const double* ang;      // (nang, 3) unit vectors
  const double* ang_w;    // (nang) weights, summing to 4 pi
  int scheme;             // 0 Becke, 1 Stratmann
  double* coords;         // (G, 3)
  double* weights;        // (G)
  long long G;
};

__global__ void __launch_bounds__(kThreads) becke_grid_kernel(const __grid_constant__ GridParams p) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < p.G;
       g += (long long)gridDim.x * blockDim.x) {
    int a = 0;
    while (a + 1 < p.natom && p.off[a + 1] <= g) ++a;
    const long long k = g - p.off[a];
    const int i = (int)(k / p.nang), j = (int)(k % p.nang);
    if (i >= p.nrad[a]) {  // offsets inconsistent with the node counts
      p.coords[3 * g] = p.coords[3 * g + 1] = p.coords[3 * g + 2] = 0.0;
      p.weights[g] = 0.0;
      continue;
    }
    const double r = p.rad_r[p.roff[a] + i];
    const double x = p.xyz[3 * a] + r * p.ang[3 * j];
    const double y = p.xyz[3 * a + 1] + r * p.ang[3 * j + 1];
    const double z = p.xyz[3 * a + 2] + r * p.ang[3 * j + 2];
    p.coords[3 * g] = x;
    p.coords[3 * g + 1] = y;
    p.coords[3 * g + 2] = z;
    double w = p.rad_w[p.roff[a] + i] * p.ang_w[j];
    if (p.natom > 1) {
      double num = 0.0, den = 0.0;
      for (int b = 0; b < p.natom; ++b) {
        const double dbx = x - p.xyz[3 * b], dby = y - p.xyz[3 * b + 1], dbz = z - p.xyz[3 * b + 2];
        const double rb = sqrt(dbx * dbx + dby * dby + dbz * dbz);
        double P = 1.0;
        for (int c = 0; c < p.natom && P > 0.0; ++c) {
          if (c == b) continue;
          const double dcx = x - p.xyz[3 * c], dcy = y - p.xyz[3 * c + 1], dcz = z - p.xyz[3 * c + 2];
          const double rc = sqrt(dcx * dcx + dcy * dcy + dcz * dcz);
          const double ex = p.xyz[3 * b] - p.xyz[3 * c], ey = p.xyz[3 * b + 1] - p.xyz[3 * c + 1],
                       ez = p.xyz[3 * b + 2] - p.xyz[3 * c + 2];
          const double mu = (rb - rc) / sqrt(ex * ex + ey * ey + ez * ez);
          const double nu = p.adj ? mu + p.adj[b * p.natom + c] * (1.0 - mu * mu) : mu;
          P *= switch_s(nu, p.scheme);
        }
        den += P;
        if (b == a) num = P;
      }
      w = den > 0.0 ? w * num / den : 0.0;
    }
    p.weights[g] = w;
  }
}

}  // namespace

extern "C" int qex_td_becke_grid(int32_t natom, const double* atom_xyz, const double* size_adjust,
                                 const int64_t* atom_point_offset, const int32_t* num_radial,
                                 const int64_t* radial_offset, const double* radial_nodes,
                                 const double* radial_weights, int32_t num_angular,
                                 const double* angular_nodes, const double* angular_weights,
                                 int32_t scheme, int64_t num_points, double* coords,
                                 double* weights, void* stream) {
  if (natom < 1 || natom > kMaxAtoms || num_angular < 1 || num_points < 0 || scheme < 0 ||
      scheme > 1)
    return QEX_BAD_ARG;
  if (!atom_xyz || !atom_point_offset || !num_radial || !radial_offset || !radial_nodes ||
      !radial_weights || !angular_nodes || !angular_weights || !coords || !weights)
    return QEX_BAD_ARG;
  if (num_points == 0) return QEX_OK;
  GridParams P{natom,        atom_xyz,     size_adjust,   atom_point_offset, num_radial,
               radial_offset, radial_nodes, radial_weights, num_angular,      angular_nodes,
               angular_weights, scheme,     coords,        weights,           num_points};
  long long blocks = (num_points + kThreads - 1) / kThreads;
  if (blocks > 65535LL * 16) blocks = 65535LL * 16;
  becke_grid_kernel<<<(unsigned)blocks, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(P);
  return cudaGetLastError() == cudaSuccess ? QEX_OK : QEX_CUDA_ERROR;
}
