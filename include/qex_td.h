/*
 * qex_td.h -- C ABI of the GB300 3D Kohn-Sham numint / generalized-eigh path.
 *
 * Device buffers, row-major, float64, caller-owned; opaque stream; int status
 * (codes of qex_ks1d.h); no allocation (workspace-size queries where needed).
 *
 * Reference interfaces replaced (qedft, pasqal-io/qex):
 *   qex_td_eval_ao        <- eval_gto 'GTOval_cart' as used at
 *                            qedft/train/td/eval_gto.py:20-70 and
 *                            qedft/train/td/scf_functions_masked.py:169-173
 *   qex_td_rho            <- eval_rho (LDA), qedft/train/td/numint_legacy.py:351-397
 *   qex_td_lda            <- eval_xc for the LDA exchange inside nr_rks,
 *                            qedft/train/td/numint_legacy.py:148-164
 *   qex_td_vxc            <- _scale_ao + _dot_ao_ao + (V + V^T),
 *                            qedft/train/td/numint_legacy.py:161-164,337,432-456
 *   qex_td_gen_eigh       <- generalized_eigh,
 *                            qedft/train/td/generalized_eigensolver.py:264-330
 *   qex_td_make_rdm1      <- make_rdm1, qedft/train/td/hf.py:303-308 and
 *                            qedft/train/td/scf_functions_masked.py:290-303
 *   qex_td_eval_ao_deriv1 <- eval_gto 'GTOval_cart_deriv1' (ao_deriv = 1 in the GGA
 *                            branch of nr_rks, qedft/train/td/numint_legacy.py:175-177)
 *   qex_td_rho_gga        <- make_rho(..., "GGA"), numint_legacy.py:180, 351-397
 *   qex_td_gga_pbe_x      <- eval_xc for a GGA functional + _rks_gga_wv0,
 *                            numint_legacy.py:181-193 (PBE exchange, restated)
 *   qex_td_vxc_gga        <- _scale_ao(ao, wv) + _dot_ao_ao + (V + V^T),
 *                            numint_legacy.py:194-196, 337
 *   qex_td_becke_grid     <- pyscf.dft.gen_grid.Grids(mol).build() with
 *                            becke_scheme = stratmann, as used at
 *                            qedft/data_io/td/dataset_generation.py:139-142
 *   qex_td_int1e          <- int1e_ovlp, int1e_kin, int1e_nuc (libcint through pyscf)
 *   qex_td_int3c2e, qex_td_int2c2e, qex_td_df_factors
 *                         <- density-fitted J, qedft/train/td/hf.py:425-449 (pyscfad
 *                            df_jk: int3c2e, int2c2e and the Cholesky-fitted factors)
 *   qex_td_fermi_occupations <- optimize_fermi_occupations /
 *                            get_fractional_occupations_jax /
 *                            get_fractional_occupations_jax_stable,
 *                            qedft/train/td/fermi.py:145-219, 301-390, 393-497
 *   qex_td_diis_error     <- get_diis_error, qedft/train/td/jax_diis.py:107-114
 *   qex_td_diis_extrapolate <- update_diis_state + extrapolate_fock,
 *                            qedft/train/td/jax_diis.py:26-104
 *   qex_td_nn_xc          <- get_exc_and_vrho, qedft/train/td/xc.py:12-47 (local MLP of
 *                            qedft/train/td/trainer_legacy_no_jit.py:56-62, 98-107)
 *   qex_td_nn_xc_global   <- exc_and_vrho_global, qedft/train/td/trainer_legacy_no_jit.py:46-53
 *   qex_td_coulomb        <- J = einsum('ijkl,kl->ij', eri, dm),
 *                            qedft/train/td/scf_functions_masked.py:152, with the
 *                            ERI in factored form (ij|kl) = sum_P B_Pij B_Pkl
 *   qex_td_fock_energy    <- get_fock without DIIS (h1e + vhf, qedft/train/td/hf.py:360-404)
 *                            fused with energy_tot (tr(D h) + 1/2 tr(D J) + E_xc + E_nuc,
 *                            qedft/train/td/scf_functions_masked.py:243-265)
 *   qex_td_orbital_gradient <- norm of mf.get_grad(mo_coeff, mo_occ, fock) (pyscf RHF
 *                            gradient 2 C_vir^T F C_occ), qedft/train/td/hf.py:81-84
 *   qex_td_scf_check      <- the stop rule |E - E_last| < conv_tol and |g| < conv_tol_grad,
 *                            qedft/train/td/hf.py:93-96 (results latched at the first
 *                            converged cycle, as the reference's loop breaks there)
 *   qex_td_aufbau_occ     <- get_occ, qedft/train/td/hf.py:602-607 and
 *                            qedft/train/td/scf_functions_masked.py:176-186
 *   qex_td_mask_pad, qex_td_mask_sort
 *                         <- the padding and slot sorting of masked_generalized_eigh,
 *                            qedft/train/td/generalized_eigensolver_masked.py:19-89
 */
#ifndef QEX_TD_H_
#define QEX_TD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shells of Cartesian contracted Gaussians: shell s has centre
 * centers[3s..3s+2], angular momentum l[s] (0, 1 or 2), primitives
 * [prim_offset[s], prim_offset[s+1]) of exponents / coefficients (the
 * coefficients include the primitive normalisation) and its first AO column
 * ao_offset[s]; its (l+1)(l+2)/2 components follow in pyscf's Cartesian order
 * (x, y, z; xx, xy, xz, yy, yz, zz), each the monomial times the radial sum.
 * A shell with l outside 0..2 is skipped (its columns are left unwritten).
 * ao is (G, nao). */
int qex_td_eval_ao(int64_t num_points, const double* coords, int32_t num_shells,
                   const double* centers, const int32_t* l, const int32_t* prim_offset,
                   const int32_t* ao_offset, const double* exponents, const double* coefficients,
                   int32_t nao, double* ao, void* stream);

/* rho_g = sum_ij ao_gi D_ij ao_gj.  workspace: qex_td_rho_workspace_size bytes. */
size_t qex_td_rho_workspace_size(int64_t num_points, int32_t nao);
int qex_td_rho(int64_t num_points, int32_t nao, const double* ao, const double* dm, double* rho,
               void* workspace, size_t workspace_bytes, void* stream);

/* Slater exchange on the grid: exc_g, vrho_g, and sums[0] = sum w rho,
 * sums[1] = sum w rho exc (deterministic). */
size_t qex_td_lda_workspace_size(int64_t num_points);
int qex_td_lda(int64_t num_points, const double* rho, const double* weights, double* exc,
               double* vrho, double* sums, void* workspace, size_t workspace_bytes, void* stream);

/* vmat = ao^T diag(0.5 w v) ao, then vmat + vmat^T.  workspace:
 * qex_td_vxc_workspace_size bytes. */
/* Slater exchange + VWN correlation (paramagnetic fit 5): the reference's
 * default "LDA,VWN" (qedft/train/td/rks.py:172).  Same arguments as qex_td_lda. */
int qex_td_lda_vwn(int64_t num_points, const double* rho, const double* weights, double* exc,
                   double* vrho, double* sums, void* workspace, size_t workspace_bytes,
                   void* stream);

size_t qex_td_vxc_workspace_size(int64_t num_points, int32_t nao);
int qex_td_vxc(int64_t num_points, int32_t nao, const double* ao, const double* weights,
               const double* vrho, double* vmat, void* workspace, size_t workspace_bytes,
               void* stream);

/* Batched generalized eigenproblem A v = w S v for `batch` matrices of order n
 * (A, S: (batch, n, n)); w (batch, n) ascending, V (batch, n, n) with the
 * eigenvectors in columns.  status (batch): 0, or QEX_NUMERICAL when S needed
 * the SPD shift and its eigenvalues were computed, or QEX_NOT_CONVERGED when
 * the Jacobi sweeps hit their cap. */
size_t qex_td_gen_eigh_workspace_size(int32_t batch, int32_t n);
int qex_td_gen_eigh(int32_t batch, int32_t n, const double* A, const double* S, double* w,
                    double* V, int32_t* status, void* workspace, size_t workspace_bytes,
                    void* stream);

/* Fermi-Dirac occupations of `batch` orbital spectra (mo_energy: (batch, n),
 * n_electrons: (batch)), by damped Newton steps on the chemical potential.
 * mode 0: stop once (N - sum occ)^2 < 1e-9, status QEX_NOT_CONVERGED when it
 * ends above 1e-2 (start mo_energy[0] + mu_shift); mode 1: min(max_steps, 100)
 * steps (same start); mode 2: start at the HOMO/LUMO midpoint, fall back to
 * theta = 0.01 when the count misses by 1e-2.  mu_initial (batch) or NULL.
 * Outputs: occ (batch, n); mu, entropic_energy (theta sum 2[f ln f +
 * (1-f) ln(1-f)]), loss and status (batch), any of these four may be NULL. */
int qex_td_fermi_occupations(int32_t batch, int32_t n, const double* mo_energy,
                             const double* n_electrons, double theta, const double* mu_initial,
                             double mu_shift, double step_grad, int32_t max_steps, int32_t mode,
                             double* occ, double* mu, double* entropic_energy, double* loss,
                             int32_t* status, void* stream);

/* GGA numint.  ao4: (4, G, nao) AO values then d/dx, d/dy, d/dz;
 * rho4: (4, G) rho then its gradient; wv: (4, G) the GGA potential weights
 * 0.5 w de/drho and 2 w de/dsigma grad rho. */
int qex_td_eval_ao_deriv1(int64_t num_points, const double* coords, int32_t num_shells,
                          const double* centers, const int32_t* l, const int32_t* prim_offset,
                          const int32_t* ao_offset, const double* exponents,
                          const double* coefficients, int32_t nao, double* ao4, void* stream);
size_t qex_td_rho_gga_workspace_size(int64_t num_points, int32_t nao);
int qex_td_rho_gga(int64_t num_points, int32_t nao, const double* ao4, const double* dm,
                   double* rho4, void* workspace, size_t workspace_bytes, void* stream);
/* PBE exchange (spin-unpolarised): exc (G, per particle; may be NULL), wv,
 * sums[0] = sum w rho, sums[1] = sum w rho exc (deterministic). */
size_t qex_td_gga_pbe_x_workspace_size(int64_t num_points);
int qex_td_gga_pbe_x(int64_t num_points, const double* rho4, const double* weights, double* exc,
                     double* wv, double* sums, void* workspace, size_t workspace_bytes,
                     void* stream);
/* vmat = M + M^T, M = ao0^T (sum_n wv_n o ao_n). */
size_t qex_td_vxc_gga_workspace_size(int64_t num_points, int32_t nao);
int qex_td_vxc_gga(int64_t num_points, int32_t nao, const double* ao4, const double* wv,
                   double* vmat, void* workspace, size_t workspace_bytes, void* stream);

/* Molecular grid: atom a contributes num_radial[a] x num_angular points
 * (atom_point_offset[a], packed atom by atom), x = R_a + r_i u_j with weight
 * w_i w_j times Becke's partition P_a / sum_b P_b.  radial_weights include
 * r^2 dr, angular_weights sum to 4 pi.  size_adjust (natom x natom) is Becke's
 * a_bc or NULL; scheme 0 Becke's switching function, 1 Stratmann's. */
int qex_td_becke_grid(int32_t natom, const double* atom_xyz, const double* size_adjust,
                      const int64_t* atom_point_offset, const int32_t* num_radial,
                      const int64_t* radial_offset, const double* radial_nodes,
                      const double* radial_weights, int32_t num_angular,
                      const double* angular_nodes, const double* angular_weights, int32_t scheme,
                      int64_t num_points, double* coords, double* weights, void* stream);

/* Gaussian integrals over Cartesian s, p and d shells (shell arrays as
 * qex_td_eval_ao, auxiliary shells likewise).  S, T, V: (nao, nao), written
 * exactly symmetric; V = -sum_C Z_C <i|1/|r - C||j>. */
int qex_td_int1e(int32_t num_shells, const double* centers, const int32_t* l,
                 const int32_t* prim_offset, const int32_t* ao_offset, const double* exponents,
                 const double* coefficients, int32_t nao, int32_t natom, const double* charges,
                 const double* positions, double* S, double* T, double* V, void* stream);
/* (ij|P): (naux, nao, nao). */
int qex_td_int3c2e(int32_t num_shells, const double* centers, const int32_t* l,
                   const int32_t* prim_offset, const int32_t* ao_offset, const double* exponents,
                   const double* coefficients, int32_t nao, int32_t num_aux_shells,
                   const double* aux_centers, const int32_t* aux_l, const int32_t* aux_prim_offset,
                   const int32_t* aux_offset, const double* aux_exponents,
                   const double* aux_coefficients, int32_t naux, double* out, void* stream);
/* (P|Q): (naux, naux). */
int qex_td_int2c2e(int32_t num_aux_shells, const double* aux_centers, const int32_t* aux_l,
                   const int32_t* aux_prim_offset, const int32_t* aux_offset,
                   const double* aux_exponents, const double* aux_coefficients, int32_t naux,
                   double* out, void* stream);
/* In place: metric (naux, naux) -> its lower Cholesky factor L; int3c
 * (naux, cols) -> L^-1 int3c.  status (device int) QEX_NUMERICAL if the
 * metric is not positive definite. */
int qex_td_df_factors(int32_t naux, int64_t cols, double* metric, double* int3c,
                      int32_t* status, void* stream);

/* D = C diag(occ) C^T for `batch` matrices (C: (batch, n, n), occ: (batch, n)). */
int qex_td_make_rdm1(int32_t batch, int32_t n, const double* C, const double* occ, double* D,
                     void* stream);

/* e = F D S - S D F (symmetric F, D, S of order n).  workspace: n*n doubles. */
int qex_td_diis_error(int32_t n, const double* F, const double* D, const double* S, double* err,
                      void* workspace, size_t workspace_bytes, void* stream);

/* CDIIS extrapolation over `nvec` stored (error, fock) pairs of n*n doubles
 * (errs, focks: (nvec, n*n), oldest first): B = [[0,-1],[-1, e_i.e_j]] + 1e-14 I,
 * solve B c = (-1, 0, ...), F = sum_i c_i F_i.  With nvec < min_vecs, F is the
 * newest stored fock.  coeffs (optional, nvec doubles) receives c. */
int qex_td_diis_extrapolate(int32_t n, int32_t nvec, int32_t min_vecs, const double* errs,
                            const double* focks, double* fock_out, double* coeffs, void* stream);

/* J_ij = sum_P B_Pij (sum_kl B_Pkl D_kl); factors (naux, n, n).
 * workspace: naux doubles. */
int qex_td_coulomb(int32_t n, int32_t naux, const double* factors, const double* dm, double* J,
                   void* workspace, size_t workspace_bytes, void* stream);

/* Neural XC on the grid: replaces get_exc_and_vrho (qedft/train/td/xc.py:12-47)
 * with the local MLP of qedft/train/td/trainer_legacy_no_jit.py:56-62, 98-107
 * (features [H, H, 1], gelu (tanh form), output -scale * swish).  rho, exc, vrho:
 * (num_points) FP64 device; params: FP32 device, w1 (H), b1 (H), W2 (H x H,
 * row = input unit), b2 (H), w3 (H), b3 (1).  exc_g = network(rho_g),
 * vrho_g = d exc_g / d rho_g; the network runs in FP32.  With weights (else
 * null, and sums null), sums = (sum w rho, sum w rho exc) in FP64 as nr_rks
 * accumulates them (qedft/train/td/numint_legacy.py:148-160). */
size_t qex_td_nn_xc_workspace_size(int64_t num_points, int32_t hidden);
int qex_td_nn_xc(int64_t num_points, int32_t hidden, const double* rho, const double* weights,
                 const float* params, double scale, double* exc, double* vrho, double* sums,
                 void* workspace, size_t workspace_bytes, void* stream);

/* Global neural XC: replaces exc_and_vrho_global (qedft/train/td/
 * trainer_legacy_no_jit.py:46-53) as consumed by the NN-AmplitudeEncoding
 * xctype of nr_rks (qedft/train/td/numint_legacy.py:311-333): the density vector
 * is one input of the MLP [H, H, 1] (W1: (num_points, H) row-major, then b1,
 * W2 (H x H), b2, w3, b3; FP32 device), exc = sum of its output (scalar),
 * vrho = d exc / d rho (num_points, FP64 device).  sums = (sum w rho, exc).
 * hidden <= 1024. */
size_t qex_td_nn_xc_global_workspace_size(int64_t num_points, int32_t hidden);
int qex_td_nn_xc_global(int64_t num_points, int32_t hidden, const double* rho,
                        const double* weights, const float* params, double scale, double* vrho,
                        double* sums, void* workspace, size_t workspace_bytes, void* stream);

/* Path of qex_td_gen_eigh for matrices of size n (1 <= n <= 240), a tuning
 * knob with no counterpart in the reference: 0 the default (FP32 solve in
 * shared memory up to n = 128, the FP64 factor and tridiagonal stage beyond),
 * 1 the shared-memory FP32 solve (n <= 128), 2 the FP64 factor and
 * tridiagonal stage.  Both are refined in FP64 to the same accuracy; the
 * faster one depends on n.  Process-wide; not synchronised with calls in
 * flight. */
int qex_td_gen_eigh_set_path(int32_t n, int32_t path);

/* F = h1e + J + V (fock may be NULL) and energy[0] = sum_ij D_ij h_ji +
 * 1/2 sum_ij D_ij J_ij + excsum[0] + energy_nuc (excsum a device scalar, may be
 * NULL for 0).  One CTA, fixed-order sums. */
int qex_td_fock_energy(int32_t n, const double* h1e, const double* J, const double* V,
                       const double* dm, const double* excsum, double energy_nuc, double* fock,
                       double* energy, void* stream);

/* norm[0] = |g|_2, g_ai = 2 (C^T F C)_ai over virtual a (mo_occ == 0 or below)
 * and occupied i (mo_occ > 0).  Workspace of the queried size. */
size_t qex_td_orbital_gradient_workspace_size(int32_t n);
int qex_td_orbital_gradient(int32_t n, const double* mo_coeff, const double* mo_occ,
                            const double* fock, double* norm, void* workspace,
                            size_t workspace_bytes, void* stream);

/* Convergence of cycle `cycle`: E = energies[cycle], E_last = energies[cycle-1]
 * (energy_init[0] for cycle 0).  state (3 ints, zeroed before cycle 0):
 * [0] converged, [1] first converged cycle, [2] cycles run up to it.  Until
 * the first converged cycle (included) the cycle's dm, mo_energy, mo_coeff,
 * mo_occ and energy are copied to the *_out buffers; after it they are left
 * alone, so the outputs are those of the cycle at which the reference's loop
 * stops, or of the last cycle when it never converges. */
int qex_td_scf_check(int32_t cycle, int32_t n, const double* energies, const double* energy_init,
                     const double* gnorm, double conv_tol, double conv_tol_grad, int32_t* state,
                     const double* dm, const double* mo_energy, const double* mo_coeff,
                     const double* mo_occ, double* dm_out, double* mo_energy_out,
                     double* mo_coeff_out, double* mo_occ_out, double* energy_out, void* stream);

/* Aufbau occupations for a batch of spectra (batch, n): 2 in the lowest
 * nelectron / 2 orbitals (ties by index), 0 elsewhere. */
int qex_td_aufbau_occ(int32_t batch, int32_t n, const double* mo_energy, int32_t nelectron,
                      double* mo_occ, void* stream);

/* Masked eigenproblem set-up and ordering (mask: n bytes, 1 = kept):
 * mask_pad writes F and S restricted to the kept block with 1e-12 on padded
 * diagonals; mask_sort orders eigenpairs by (mask ? w : 1e12), stably, zeroes
 * the padded eigenvalues and the padded rows and columns of V. */
int qex_td_mask_pad(int32_t n, const double* fock, const double* s1e, const uint8_t* mask,
                    double* fock_out, double* s1e_out, void* stream);
int qex_td_mask_sort(int32_t n, const double* w, const double* V, const uint8_t* mask,
                     double* w_out, double* V_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QEX_TD_H_ */
