"""Drop-in for ``qedft/train/od/scf.py`` on the GB300 kernels.

Same names, argument meaning and defaults as the reference module.  The XC
callable must be a qex_gb300 functional (see ``qex_gb300.xc``), the
interaction one of ``qex_gb300.od.utils.exponential_coulomb`` /
``soft_coulomb``.  Results are host NumPy arrays, as the reference returns
``jnp`` arrays; batched device-resident solves live in ``qex_gb300.od.engine``.

Extra keyword (not in the reference): ``stencil`` (5, the jax_dft
fourth-order Laplacian the reference uses, or 3).
"""

from __future__ import annotations

import typing

import numpy as np

from .. import _native as N
from . import utils
from .engine import Molecule1D, PackedBatch, SolveConfig, default_engine
from .xc_eval import xc_energy_and_potential


class KohnShamState(typing.NamedTuple):
    """jax_dft ``scf.KohnShamState`` (fields used at ``qedft/train/od/jit_scf.py:214-234``)."""

    density: np.ndarray
    total_energy: typing.Any
    locations: np.ndarray
    nuclear_charges: np.ndarray
    external_potential: np.ndarray
    grids: np.ndarray
    num_electrons: typing.Any
    hartree_potential: typing.Any = None
    xc_potential: typing.Any = None
    xc_energy_density: typing.Any = None
    gap: typing.Any = None
    converged: typing.Any = False


def get_xc_energy_amplitude_encoded(density, xc_energy_density_fn, grids):
    """E_xc = dx * sum f(n) (``qedft/train/od/scf.py:32-50``), on the GPU."""
    e, _, _ = xc_energy_and_potential(density, xc_energy_density_fn, grids, "amplitude")
    return e


def get_xc_potential_amplitude_encoded(density, xc_energy_density_fn, grids):
    """v_xc = dE_xc/dn, including the factor dx (``qedft/train/od/scf.py:53-76``)."""
    _, v, _ = xc_energy_and_potential(density, xc_energy_density_fn, grids, "amplitude")
    return v


def _molecule(state_or_args, grids, locations, charges, num_electrons, **kw):
    return Molecule1D.from_grids(grids, locations, charges, num_electrons, **kw)


def _iteration(state, num_electrons, xc_energy_density_fn, interaction_fn,
               enforce_reflection_symmetry, convention, stencil):
    torch = N.require_cuda()
    grids = np.asarray(state.grids, dtype=np.float64)
    mol = _molecule(state, grids, state.locations, state.nuclear_charges, int(num_electrons))
    batch = PackedBatch([mol], sort=False)
    cfg = SolveConfig(num_iterations=1, enforce_reflection_symmetry=enforce_reflection_symmetry,
                      convention=convention, stencil=stencil, interaction=interaction_fn)
    dens = torch.as_tensor(np.asarray(state.density, np.float64), device=batch.device)
    vext = torch.as_tensor(np.asarray(state.external_potential, np.float64), device=batch.device)
    out = default_engine().iteration(batch, xc_energy_density_fn, cfg, dens, vext)
    torch.cuda.current_stream().synchronize()
    f = out["xc_energy_density"].cpu().numpy()
    xced = float(np.sum(f)) if convention == "amplitude" else f
    return state._replace(
        density=out["density"].cpu().numpy(),
        total_energy=float(out["energy"].cpu().numpy()[0, 0]),
        hartree_potential=out["hartree_potential"].cpu().numpy(),
        xc_potential=out["xc_potential"].cpu().numpy(),
        xc_energy_density=xced,
        gap=float(out["gap"].cpu().numpy()[0, 0]),
    )


def kohn_sham_iteration_amplitude_encoded(state, num_electrons, xc_energy_density_fn,
                                          interaction_fn, enforce_reflection_symmetry, *,
                                          stencil=5):
    """One KS iteration (``qedft/train/od/scf.py:79-177``)."""
    return _iteration(state, num_electrons, xc_energy_density_fn, interaction_fn,
                      enforce_reflection_symmetry, "amplitude", stencil)


def _stack_states(out, batch, mol, cfg, convention, grids):
    torch = N.require_cuda()
    torch.cuda.current_stream().synchronize()
    T = cfg.num_iterations
    n = mol.num_grids
    host = {k: v.cpu().numpy() for k, v in out.items()}
    f = host["xc_energy_density"].reshape(T, n)
    xced = f.sum(axis=1) if convention == "amplitude" else f
    status = int(host["status"][0])
    if status & 0xff:
        raise RuntimeError(f"SCF kernel reported status {status}")
    return KohnShamState(
        density=host["density"].reshape(T, n),
        total_energy=host["energy"][0],
        locations=np.tile(mol.locations, (T, 1)),
        nuclear_charges=np.tile(mol.nuclear_charges, (T, 1)),
        external_potential=np.tile(host["external_potential"], (T, 1)),
        grids=np.tile(grids, (T, 1)),
        num_electrons=np.full(T, mol.num_electrons),
        hartree_potential=host["hartree_potential"].reshape(T, n),
        xc_potential=host["xc_potential"].reshape(T, n),
        xc_energy_density=xced,
        gap=host["gap"][0],
        converged=host["converged"][0].astype(bool),
    )


def run_scf(locations, nuclear_charges, num_electrons, num_iterations, grids, xc_energy_density_fn,
            interaction_fn, initial_density, alpha, alpha_decay, enforce_reflection_symmetry,
            num_mixing_iterations, density_mse_converge_tolerance, rule, convention, stencil):
    grids = np.asarray(grids, dtype=np.float64)
    mol = Molecule1D.from_grids(grids, locations, nuclear_charges, int(num_electrons),
                                initial_density=None if initial_density is None
                                else np.asarray(initial_density, np.float64))
    batch = PackedBatch([mol], sort=False)
    cfg = SolveConfig(num_iterations=int(num_iterations), alpha=alpha, alpha_decay=alpha_decay,
                      num_mixing_iterations=int(num_mixing_iterations),
                      density_mse_converge_tolerance=float(density_mse_converge_tolerance),
                      enforce_reflection_symmetry=bool(enforce_reflection_symmetry),
                      convergence_rule=rule, convention=convention, stencil=stencil,
                      interaction=interaction_fn)
    out = default_engine().solve(batch, xc_energy_density_fn, cfg)
    return _stack_states(out, batch, mol, cfg, convention, grids)


def kohn_sham_amplitude_encoded(locations, nuclear_charges, num_electrons, num_iterations, grids,
                                xc_energy_density_fn, interaction_fn, initial_density=None,
                                alpha=0.5, alpha_decay=0.9, enforce_reflection_symmetry=False,
                                num_mixing_iterations=2, density_mse_converge_tolerance=-1.0, *,
                                stencil=5):
    """SCF with the Python-loop rules of ``qedft/train/od/scf.py:434-560``: default
    initial density = non-interacting solution, converged = MSE(unmixed - old) < tol,
    early stop pads with the converged state."""
    return run_scf(locations, nuclear_charges, num_electrons, num_iterations, grids,
                   xc_energy_density_fn, interaction_fn, initial_density, alpha, alpha_decay,
                   enforce_reflection_symmetry, num_mixing_iterations,
                   density_mse_converge_tolerance, "python", "amplitude", stencil)


kohn_sham_amplitude_encoded_no_jit = kohn_sham_amplitude_encoded


def solve_noninteracting_system(external_potential, num_electrons, grids, *, stencil=5):
    """(density, total_eigen_energies, gap) of T + diag(v) (``qedft/train/od/scf.py:233-250``)."""
    torch = N.require_cuda()
    grids = np.asarray(grids, dtype=np.float64)
    mol = Molecule1D.from_grids(grids, [0.0], [0.0], int(num_electrons))
    batch = PackedBatch([mol], sort=False)
    v = torch.as_tensor(np.asarray(external_potential, np.float64), device=batch.device)
    dens, tee, gap, status = default_engine().noninteracting(batch, v, stencil=stencil)
    torch.cuda.current_stream().synchronize()
    return dens.cpu().numpy(), float(tee.cpu()[0]), float(gap.cpu()[0])
