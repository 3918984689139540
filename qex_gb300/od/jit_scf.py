"""Drop-in for ``qedft/train/od/jit_scf.py`` (and jax_dft ``jit_scf.kohn_sham``).

``kohn_sham_amplitude_encoded`` keeps the signature of
``qedft/train/od/jit_scf.py:247-330`` (lax.scan rules: converged-skip,
connection-weight mixing, converged = MSE(mixed - old) < tol, alpha decays
every step).  ``kohn_sham`` is the local-XC twin selected at
``qedft/train/od/train.py:117-121``.  ``stop_gradient_step`` only affects
gradients; the forward pass ignores it (see ``qex_gb300.od.adjoint``).
"""

from __future__ import annotations

from .scf import KohnShamState, _iteration, run_scf


def kohn_sham_iteration_amplitude_encoded(state, num_electrons, xc_energy_density_fn,
                                          interaction_fn, enforce_reflection_symmetry, *,
                                          stencil=5):
    """``qedft/train/od/jit_scf.py:89-140``."""
    return _iteration(state, num_electrons, xc_energy_density_fn, interaction_fn,
                      enforce_reflection_symmetry, "amplitude", stencil)


def kohn_sham_iteration(state, num_electrons, xc_energy_density_fn, interaction_fn,
                        enforce_reflection_symmetry, *, stencil=5):
    """jax_dft ``jit_scf.kohn_sham_iteration`` (local XC convention)."""
    return _iteration(state, num_electrons, xc_energy_density_fn, interaction_fn,
                      enforce_reflection_symmetry, "local", stencil)


def kohn_sham_amplitude_encoded(locations, nuclear_charges, num_electrons, num_iterations, grids,
                                xc_energy_density_fn, interaction_fn, initial_density,
                                alpha=0.5, alpha_decay=0.9, enforce_reflection_symmetry=False,
                                num_mixing_iterations=2, density_mse_converge_tolerance=-1.0,
                                stop_gradient_step=-1, *, stencil=5) -> KohnShamState:
    del stop_gradient_step
    if initial_density is None:
        raise ValueError("the jit-able SCF requires initial_density (qedft/train/od/jit_scf.py:268)")
    return run_scf(locations, nuclear_charges, num_electrons, num_iterations, grids,
                   xc_energy_density_fn, interaction_fn, initial_density, alpha, alpha_decay,
                   enforce_reflection_symmetry, num_mixing_iterations,
                   density_mse_converge_tolerance, "jit", "amplitude", stencil)


def kohn_sham(locations, nuclear_charges, num_electrons, num_iterations, grids,
              xc_energy_density_fn, interaction_fn, initial_density, alpha=0.5, alpha_decay=0.9,
              enforce_reflection_symmetry=False, num_mixing_iterations=2,
              density_mse_converge_tolerance=-1.0, stop_gradient_step=-1, *,
              stencil=5) -> KohnShamState:
    """jax_dft ``jit_scf.kohn_sham`` semantics with the local XC convention."""
    del stop_gradient_step
    if initial_density is None:
        raise ValueError("the jit-able SCF requires initial_density")
    return run_scf(locations, nuclear_charges, num_electrons, num_iterations, grids,
                   xc_energy_density_fn, interaction_fn, initial_density, alpha, alpha_decay,
                   enforce_reflection_symmetry, num_mixing_iterations,
                   density_mse_converge_tolerance, "jit", "local", stencil)
