/*
 * qex_xc1d.h -- point-parallel evaluation of the 1D XC functionals.
 *
 * Reference interfaces replaced (qedft, pasqal-io/qex):
 *   qex_xc1d_eval <- get_xc_energy_amplitude_encoded and
 *                    get_xc_potential_amplitude_encoded,
 *                    qedft/train/od/scf.py:32-76 (the potential is dE/dn and
 *                    carries the factor dx), and the jax_dft local-convention
 *                    get_xc_energy / get_xc_potential used through
 *                    qedft/train/od/train.py:117-121.
 *
 * Densities are packed as in qex_ks1d.h (molecule b at grid_offsets[b]).
 * Outputs (any may be NULL): per-point values f (packed), v_xc (packed) and
 * E_xc per molecule.  The window MLP needs a workspace of
 * qex_xc1d_workspace_size(total_points) bytes, total_points >= every
 * grid_offsets[b] + num_grids[b].
 *
 *   qex_ksr1d_eval <- the KSR functional's xc_energy_density_fn(density, params)
 *                    and its gradient (qedft/models/classical/global_ksr_model.py:32-80,
 *                    jax_dft neural_xc.global_functional), evaluated per
 *                    molecule on its own grid.  Same outputs; one warp per
 *                    molecule, no workspace (shared memory sized by
 *                    max_num_grids >= every num_grids[b]).
 */
#ifndef QEX_XC1D_H_
#define QEX_XC1D_H_

#include <stddef.h>
#include <stdint.h>

#include "qex_ks1d.h"

#ifdef __cplusplus
extern "C" {
#endif

int qex_xc1d_workspace_size(int64_t total_points, const qex_xc_spec* xc, size_t* bytes);

int qex_xc1d_eval(int32_t num_molecules, int64_t total_points, const int32_t* num_grids,
                  const int64_t* grid_offsets, const double* grid_spacing,
                  const qex_xc_spec* xc, const double* density, double* values,
                  double* potential, double* energy, void* workspace, size_t workspace_bytes,
                  void* stream);

int qex_ksr1d_eval(int32_t num_molecules, int32_t max_num_grids, const int32_t* num_grids,
                   const int64_t* grid_offsets, const double* grid_spacing,
                   const qex_xc_spec* xc, const double* density, double* values,
                   double* potential, double* energy, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QEX_XC1D_H_ */
