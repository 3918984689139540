/*
 * qex_ks1d.h -- C ABI of the GB300 1D Kohn-Sham SCF path.
 *
 * Every entry point works on caller-owned DEVICE buffers (row-major, batch
 * first, float64 unless stated), takes the CUDA stream as an opaque pointer,
 * allocates nothing and returns an int status (QEX_OK on success).  Molecules
 * of different grid sizes are packed one after another: molecule b's grid
 * vectors start at element grid_offsets[b] of every packed array and hold
 * num_grids[b] values.  Per-iteration records of molecule b start at element
 * num_iterations * grid_offsets[b] and are (num_iterations, num_grids[b]).
 *
 * Reference interfaces replaced (qedft, pasqal-io/qex):
 *   qex_ks1d_solve      <- qedft/train/od/jit_scf.py:247-330
 *                          (kohn_sham_amplitude_encoded, lax.scan form),
 *                          qedft/train/od/scf.py:434-560 (Python-loop form),
 *                          jax_dft jit_scf.kohn_sham as selected at
 *                          qedft/train/od/train.py:117-121, and the
 *                          jax.vmap batch of qedft/train/od/train.py:125.
 *   qex_ks1d_iteration  <- qedft/train/od/jit_scf.py:89-140
 *                          (kohn_sham_iteration_amplitude_encoded) and
 *                          qedft/train/od/scf.py:79-177.
 *   qex_ks1d_noninteracting <- solve_noninteracting_system as called at
 *                          qedft/train/od/scf.py:233-250,499-504.
 */
#ifndef QEX_KS1D_H_
#define QEX_KS1D_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (returned, and per molecule in `status`). */
#define QEX_OK 0
#define QEX_BAD_ARG 1
#define QEX_NOT_CONVERGED 2
#define QEX_NUMERICAL 3
#define QEX_OOM 4
#define QEX_TIMEOUT 5
#define QEX_CUDA_ERROR 6

/* Per-molecule status flags OR-ed into `status` (bit 8 and up). */
#define QEX_FLAG_DEGENERATE_FRONTIER 0x100 /* HOMO/LUMO closer than the FP32 resolution */
#define QEX_FLAG_REFINE_CAP 0x200          /* eigenpair refinement hit its step cap */

#define QEX_KS1D_MAX_EIGENPAIRS 16 /* floor(Ne/2)+1 <= 16, i.e. Ne <= 30 */
#define QEX_MLP_WINDOW 17
#define QEX_MLP_HIDDEN 16
/* W1 (17x16), b1 (16), W2 (16x16), b2 (16), W3 (16), b3 (1), as x@W+b. */
#define QEX_MLP_NUM_PARAMS (17 * 16 + 16 + 16 * 16 + 16 + 16 + 1)

/* Global-local convolutional KSR network (qedft/models/classical/global_ksr_model.py:32-80,
 * jax_dft neural_xc) with C = 16 (the reference default) or 8 channels: the
 * density and C - 1 exponential global convolutions, two bias-free width-3
 * convolutions C -> C with swish, a width-1 convolution C -> 1, -swish, and
 * the self-interaction layer.  Packed FP32 layout, QEX_KSR_NUM_PARAMS(C)
 * floats in a DEVICE buffer, 16-byte aligned:
 *   W1[t][c][o] (3 C C; tap t applies to the point at offset t - 1),
 *   W2[t][c][o] (3 C C), W3[c] (C),
 *   eta (C - 1): widths minval + (maxval - minval) * sigmoid(eta),
 *   the self-interaction width (1).
 * The network is staged into a constant-memory slot per call, so a KSR call
 * (qex_ks1d_solve* or qex_ksr1d_eval) on a stream that is being captured into
 * a CUDA graph is refused with QEX_BAD_ARG. */
#define QEX_KSR_CHANNELS 16
#define QEX_KSR_NUM_PARAMS(c) (6 * (c) * (c) + 2 * (c))

enum qex_interaction_kind {
  QEX_INTERACTION_EXPONENTIAL = 0, /* a * exp(-b |d|), jax_dft exponential_coulomb */
  QEX_INTERACTION_SOFT_COULOMB = 1 /* 1 / sqrt(d^2 + a), jax_dft soft_coulomb */
};

enum qex_xc_kind {
  QEX_XC_NONE = 0,
  QEX_XC_LDA_EXP_COULOMB = 1, /* exponential-Coulomb uniform-gas LDA */
  QEX_XC_POWER = 2,           /* f(n) = coefficient * (n + shift)^power */
  QEX_XC_WINDOW_MLP = 3,      /* FP32 window-17 MLP, two SiLU layers of 16 */
  QEX_XC_KSR = 4,             /* FP32 global-local conv network (whole-grid functional) */
  QEX_XC_LOCAL_MLP = 5,       /* FP32 dense network per grid point (LocalMLP) */
  QEX_XC_GLOBAL_MLP = 6       /* FP32 dense network on the whole density (GlobalMLP) */
};

/* Dense XC networks of qedft/models/networks.py:83-138 (LocalMLP, GlobalMLP;
 * stax stacks of qedft/models/classical/classical_models.py:77-224):
 *   x -> [Dense(H), activation] x L -> Dense(1),  x = n / normalization,
 * with x = n_i per grid point (local) or the whole density (global, whose
 * input size is nn_inputs = the grid size of every molecule).  The wrappers of
 * qedft/models/wrappers.py:162-217 are flags: QEX_NN_SELF_INTERACTION
 * (u_i = beta (-v_H[n]_i / 2) + (1 - beta) g_i, beta = exp(-((dx sum n - 1) /
 * width)^2), v_H with the default exponential Coulomb interaction) and
 * QEX_NN_NEGATIVITY (f = -swish(u)); a global network's values are its mean
 * over the grid (per-point values f_i / N).  Packed FP32 parameters in a
 * DEVICE buffer, 16-byte aligned, hidden width padded to Hp = nn_width (a
 * multiple of 8, at most 128) with zero weights: W1 (nn_inputs x Hp), b1 (Hp),
 * then per further hidden layer W (Hp x Hp), b (Hp), then Wout (Hp), then
 * {bout, width, 0, 0}: QEX_NN_NUM_PARAMS floats.  The network runs in FP32,
 * the wrappers and sums in FP64.  Neither has an adjoint step. */
enum qex_nn_activation {
  QEX_NN_TANH = 0,
  QEX_NN_RELU = 1,
  QEX_NN_SOFTPLUS = 2,
  QEX_NN_SIGMOID = 3,
  QEX_NN_ELU = 4,
  QEX_NN_LEAKY_RELU = 5, /* negative slope 0.01 */
  QEX_NN_SELU = 6,
  QEX_NN_GELU = 7        /* tanh approximation */
};
#define QEX_NN_SELF_INTERACTION 1
#define QEX_NN_NEGATIVITY 2
#define QEX_NN_MAX_WIDTH 128
#define QEX_NN_NUM_PARAMS(inputs, hp, layers) \
  ((inputs) * (hp) + (hp) + ((layers) - 1) * ((hp) * (hp) + (hp)) + (hp) + 4)

enum qex_xc_convention {
  QEX_XC_AMPLITUDE = 0, /* qedft: E = dx sum f, v = dE/dn (scf.py:32-76) */
  QEX_XC_LOCAL = 1      /* jax_dft: E = dx sum f n, v = (dE/dn)/dx */
};

typedef struct qex_xc_spec {
  int32_t kind;       /* enum qex_xc_kind */
  int32_t convention; /* enum qex_xc_convention */
  double coefficient, power, shift; /* QEX_XC_POWER */
  double lda_amplitude, lda_kappa;  /* QEX_XC_LDA_EXP_COULOMB */
  double normalization;             /* QEX_XC_WINDOW_MLP input divisor */
  const float* mlp_params_host;     /* HOST pointer, QEX_MLP_NUM_PARAMS floats */
  const float* ksr_params;          /* DEVICE pointer, QEX_KSR_NUM_PARAMS(ksr_channels) floats */
  double ksr_minval, ksr_maxval;    /* range of the global-convolution widths */
  int32_t ksr_channels;             /* 16 or 8 (QEX_XC_KSR) */
  const float* nn_params;           /* DEVICE pointer, QEX_NN_NUM_PARAMS floats (LOCAL/GLOBAL_MLP) */
  int32_t nn_width;                 /* padded hidden width Hp: multiple of 8, <= 128 */
  int32_t nn_layers;                /* hidden layers L >= 1 */
  int32_t nn_activation;            /* enum qex_nn_activation */
  int32_t nn_inputs;                /* 1 (local) or the grid size (global) */
  int32_t nn_flags;                 /* QEX_NN_SELF_INTERACTION | QEX_NN_NEGATIVITY */
  /* QEX_XC_WINDOW_MLP only: a DEVICE pointer to the same QEX_MLP_NUM_PARAMS
   * parameters in FP64 (16-byte aligned), or NULL.  Given, the network runs in
   * FP64 in the SCF and in the adjoint step: a checking mode in which the
   * adjoint's gradient can be compared with finite differences without the
   * FP32 network's rounding.  mlp_params_host must still be given. */
  const double* mlp_params64;
} qex_xc_spec;

typedef struct qex_ks1d_options {
  int32_t stencil;     /* 3 or 5 point kinetic operator */
  int32_t interaction; /* enum qex_interaction_kind */
  double interaction_a, interaction_b;
  int32_t num_iterations;
  double alpha, alpha_decay;
  int32_t num_mixing_iterations;
  double density_mse_converge_tolerance;
  int32_t convergence_rule;            /* 0: jit scan rule, 1: Python-loop rule */
  int32_t enforce_reflection_symmetry; /* flip-average about the grid centre */
  int32_t external_potential_given;    /* 1: read external_potential instead of nuclei */
  int32_t max_num_grids;               /* upper bound on num_grids[b] */
  int32_t max_num_electrons;           /* upper bound on num_electrons[b] */
  int32_t max_nuclei;                  /* row stride of locations / nuclear_charges */
  int32_t solve_planes; /* FP32 solve planes: 0 automatic (resident when the batch fits in
                           one wave of resident warps), 1 resident in shared memory,
                           2 streamed through a shared-memory ring (more warps per SM;
                           for large batches, or several batches launched concurrently) */
  int32_t solve_chunk;  /* points per chunk of the streamed planes' ring: 0 (default 32),
                           16, 32 or 64 (a tile shape the launch-plan autotuner picks) */
} qex_ks1d_options;

/* Molecule descriptors: all device arrays of length num_molecules (nuclei:
 * num_molecules * max_nuclei).  The grid of molecule b is
 * grid_start[b] + i * grid_spacing[b], i < num_grids[b]. */
typedef struct qex_ks1d_batch {
  int32_t num_molecules;
  const int32_t* num_grids;
  const int64_t* grid_offsets;
  const double* grid_start;
  const double* grid_spacing;
  const int32_t* num_electrons;
  const int32_t* num_nuclei;
  const double* locations;
  const double* nuclear_charges;
  const double* external_potential; /* packed, used if external_potential_given */
  const double* initial_density;    /* packed, or NULL: non-interacting start */
  const int32_t* order;             /* processing order (a permutation), or NULL */
} qex_ks1d_batch;

/* Outputs; any pointer may be NULL to skip that record. */
typedef struct qex_ks1d_outputs {
  double* total_energy;      /* (B, iters) */
  double* gap;               /* (B, iters) */
  uint8_t* converged;        /* (B, iters) */
  double* density;           /* per-iteration records (mixed density) */
  double* hartree_potential; /* per-iteration records */
  double* xc_potential;      /* per-iteration records */
  double* xc_energy_density; /* per-iteration records: per-point f (or eps) */
  double* final_density;     /* packed (sum N) */
  double* external_potential_out; /* packed (sum N) */
  int32_t* status;           /* (B) */
  int32_t* iterations_run;   /* (B) iterations that did work (not skipped as converged) */
  int32_t* stats;            /* (B, 8): eigen-solves, Rayleigh-quotient vector passes,
                                correction updates, Sturm multisection passes,
                                warm-route attempts, warm-route fallbacks to
                                the cold route, 2 reserved */
  int64_t* phase_cycles;     /* (B, 16): SM clock cycles per phase: Hartree, XC potential,
                                Sturm brackets, FP32 inverse iteration, FP64 refinement,
                                density+energy, mixing+records, whole molecule; then
                                parts of those: start vectors, FP32 factorisation,
                                FP32 solves (inverse iteration), Rayleigh quotients and
                                residuals, FP32 correction solves, FP64 updates, XC
                                energy, cluster Rayleigh-Ritz + normalisation */
} qex_ks1d_outputs;

/* Bytes of device workspace qex_ks1d_solve needs for this batch shape. */
int qex_ks1d_workspace_size(const qex_ks1d_options* options, int32_t num_molecules,
                            size_t* bytes);

/* Workspace for this batch shape and functional.  With a KSR functional it
 * adds num_molecules x num_iterations x max_num_grids doubles: given that
 * much, qex_ks1d_solve evaluates the network on the output densities (the
 * E_xc term of the recorded total energies) in one batched launch after the
 * SCF instead of inside it.  Same results; no counterpart in the reference
 * (its scan evaluates E_xc inside each iteration, jit_scf.py:46-72). */
int qex_ks1d_workspace_size_xc(const qex_ks1d_options* options, const qex_xc_spec* xc,
                               int32_t num_molecules, size_t* bytes);

/* Full SCF for a batch of molecules in one launch (one warp per molecule,
 * persistent CTAs, all iterations inside the kernel). */
int qex_ks1d_solve(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                   const qex_xc_spec* xc, const qex_ks1d_outputs* outputs,
                   void* workspace, size_t workspace_bytes, void* stream);

/* qex_ks1d_solve without a workspace argument and without any allocation.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc at solve time -- code running inside another framework's device
 * memory pool (an XLA custom call with no workspace reserved, a serving loop
 * whose memory is budgeted up front) or a runtime that forbids allocation on
 * its hot path.  Its scratch is a fixed 16 MiB device array inside this
 * library; a batch whose qex_ks1d_workspace_size exceeds 16 MiB is rejected
 * with QEX_OOM before anything is launched.  Each call outside stream
 * capture looks up the array's device address on the current device
 * (cudaGetSymbolAddress), which stays valid across a device reset; a call
 * under capture reuses the address of the last call outside capture, so make
 * the first call on each device before any stream capture.  Every call shares the one array:
 * calls that overlap on the GPU (other streams, other host threads) race and
 * corrupt each other's results; serialise them.  The array keeps the last
 * call's contents; what must start at zero (the work counter) is cleared by
 * each call. */
int qex_ks1d_solve_static(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                          const qex_xc_spec* xc, const qex_ks1d_outputs* outputs, void* stream);

/* One Kohn-Sham iteration per molecule: input density (packed) and external
 * potential (packed) -> unmixed output density, energy, v_H, v_xc, f, gap.
 * Records are single-iteration (iters = 1). */
int qex_ks1d_iteration(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                       const qex_xc_spec* xc, const double* density_in,
                       const qex_ks1d_outputs* outputs, void* workspace,
                       size_t workspace_bytes, void* stream);

/* Non-interacting ground state of T + diag(v) for each molecule:
 * density (packed), total eigen-energy (B) and gap (B). */
int qex_ks1d_noninteracting(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                            const double* potential, double* density,
                            double* total_eigen_energy, double* gap, int32_t* status,
                            void* workspace, size_t workspace_bytes, void* stream);

/* Reverse-mode step of one SCF iteration t (the adjoint of
 * qedft/train/od/jit_scf.py:184-211 with the local convention, as
 * differentiated by jax.value_and_grad at qedft/train/od/trainer.py:139-143).
 * Inputs: the iteration's input density n_t (packed), the upstream gradient
 * with respect to the mixed output density n_{t+1} (packed), the upstream
 * gradient with respect to this iteration's energy (B; NULL = 0) and its
 * mixing factor alpha_t.  Outputs: the gradient with respect to n_t (packed)
 * and, ACCUMULATED into grad_params (B, QEX_MLP_NUM_PARAMS), the gradient
 * with respect to the window-MLP parameters.  Window-MLP XC in the local
 * convention, exponential interaction, one mixing difference; reflection
 * symmetry (enforce_reflection_symmetry) on or off. */
int qex_ks1d_adjoint_workspace_size(const qex_ks1d_options* options, int32_t num_molecules,
                                    size_t* bytes);
int qex_ks1d_adjoint_step(const qex_ks1d_batch* batch, const qex_ks1d_options* options,
                          const qex_xc_spec* xc, const double* density_in,
                          const double* grad_density_next, const double* grad_energy,
                          double alpha, double* grad_density, double* grad_params,
                          int32_t* status, void* workspace, size_t workspace_bytes,
                          void* stream);

/* Library version string and the number of kernel launches the last call on
 * this host thread issued (for launch accounting in benchmarks). */
const char* qex_version(void);
int qex_last_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* QEX_KS1D_H_ */
