"""Seeded synthetic 3D molecules with the shapes of the 3D numint configuration.

pyscf is not available here, so one- and two-electron integrals come from a
documented synthetic model built on the molecule's own grid:

* atoms H/C/N/O at random positions with a minimum separation of 1.0 Angstrom;
* basis: Cartesian contracted Gaussians, H: 2 s shells; C, N, O: 3 s + 2 p
  shells (1-3 primitives, exponents log-uniform in [0.1, 50]); with
  ``basis="spd"`` C, N, O also carry one d shell (6 Cartesian components, one
  primitive, exponent log-uniform in [0.3, 3]);
* grid: points drawn from Gaussian clouds around the atoms, with Monte-Carlo
  importance weights 1 / (G p(r)) times a random factor in [0.9, 1.1]
  (positive random weights); or, with ``grid="becke"``, the Becke/Stratmann
  molecular grid of ``qex_gb300.td.grids`` at ``level`` (built on the GPU),
  on which the quadratures below are accurate;
* S = ao^T W ao, T = 1/2 sum_c (d_c ao)^T W (d_c ao),
  V = -ao^T diag(w sum_A Z_A / sqrt(|r - R_A|^2 + 0.2)) ao, h1e = T + V;
* two-electron integrals in factored form (ij|kl) = sum_P B_Pij B_Pkl with
  naux = 3 nao Gaussian auxiliary functions g_P on random atoms,
  B_P = 0.3 ao^T diag(w g_P) ao;
* E_nuc = sum_{A<B} Z_A Z_B / R_AB; an even electron count (sum Z, minus one
  if odd).
This is generation of inputs (host NumPy, once per molecule), not the SCF
hot path.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

ELEMENTS = {"H": 1, "C": 6, "N": 7, "O": 8}
ANGSTROM = 1.8897261246


@dataclasses.dataclass
class Shell:
    center: np.ndarray
    l: int
    exponents: np.ndarray
    coefficients: np.ndarray


@dataclasses.dataclass
class Molecule3D:
    charges: np.ndarray
    positions: np.ndarray
    shells: list
    coords: np.ndarray
    weights: np.ndarray
    nelectron: int
    ao: np.ndarray | None = None
    s1e: np.ndarray | None = None
    h1e: np.ndarray | None = None
    eri_factors: np.ndarray | None = None
    energy_nuc: float = 0.0

    @property
    def nao(self):
        return sum(ncart(s.l) for s in self.shells)

    def shell_arrays(self):
        """Flattened shell description for ``qex_td_eval_ao``."""
        return shell_arrays(self.shells)


MAX_L = 2  # s, p and d shells


def ncart(l):
    """Cartesian components of a shell of angular momentum l."""
    return (l + 1) * (l + 2) // 2


def cart_components(l):
    """(i, j, k) exponents of the components, pyscf's Cartesian order."""
    return [(i, l - i - k, k) for i in range(l, -1, -1) for k in range(0, l - i + 1)]


def shell_arrays(shells):
    """(centers, l, prim_offset, ao_offset, exponents, coefficients) of a shell
    list, as the GPU entry points take them; ValueError for l outside 0..2."""
    bad = [s.l for s in shells if not 0 <= int(s.l) <= MAX_L]
    if bad:
        raise ValueError(f"shells with l = {bad[0]}: only s, p and d shells are supported")
    centers = np.array([s.center for s in shells], dtype=np.float64).reshape(-1)
    l = np.array([s.l for s in shells], dtype=np.int32)
    poff = np.zeros(len(shells) + 1, dtype=np.int32)
    poff[1:] = np.cumsum([len(s.exponents) for s in shells])
    aoff = np.zeros(len(shells), dtype=np.int32)
    aoff[1:] = np.cumsum([ncart(s.l) for s in shells])[:-1]
    ex = np.concatenate([s.exponents for s in shells]).astype(np.float64)
    co = np.concatenate([s.coefficients for s in shells]).astype(np.float64)
    return centers, l, poff, aoff, ex, co


def _prim_norm(alpha, l):
    return (2.0 * alpha / math.pi) ** 0.75 * (4.0 * alpha) ** (0.5 * l)


def ao_values(shells, coords, deriv=False):
    """Host AO values (and gradients) for the integral model."""
    G = coords.shape[0]
    n = sum(ncart(s.l) for s in shells)
    ao = np.zeros((G, n))
    grad = np.zeros((3, G, n)) if deriv else None
    k = 0
    for s in shells:
        d = coords - s.center[None, :]
        r2 = np.einsum("gc,gc->g", d, d)
        e = np.exp(-np.outer(r2, s.exponents))
        rad = e @ s.coefficients
        drad = e @ (-2.0 * s.exponents * s.coefficients)
        for c in cart_components(s.l):
            mono = d[:, 0] ** c[0] * d[:, 1] ** c[1] * d[:, 2] ** c[2]
            ao[:, k] = mono * rad
            if deriv:
                for q in range(3):
                    dm = 0.0
                    if c[q]:
                        e_q = list(c)
                        e_q[q] -= 1
                        dm = c[q] * d[:, 0] ** e_q[0] * d[:, 1] ** e_q[1] * d[:, 2] ** e_q[2]
                    grad[q, :, k] = dm * rad + mono * drad * d[:, q]
            k += 1
    return (ao, grad) if deriv else ao


def analytic_integrals(mol: Molecule3D) -> Molecule3D:
    """Replace the model integrals by analytic ones computed on the GPU
    (``qex_gb300.td.integrals``): S, h1e = T + V_nuc, and density-fitted
    Coulomb factors over an even-tempered auxiliary basis."""
    from . import integrals

    S, T, V = integrals.int1e(mol)
    B = integrals.df_factors(mol)
    mol.s1e = S.cpu().numpy()
    mol.h1e = (T + V).cpu().numpy()
    mol.eri_factors = B.cpu().numpy()
    return mol


def synthetic_molecule(num_atoms: int, seed: int = 0, points_per_atom: int = 620,
                       with_integrals: bool = True, grid: str = "cloud",
                       level: int = 3, integrals: str = "model",
                       basis: str = "sp") -> Molecule3D:
    """``integrals``: "model" (the documented quadrature model above) or
    "analytic" (Gaussian integrals and density fitting on the GPU).
    ``basis``: "sp" or "spd" (a d shell on C, N, O)."""
    if basis not in ("sp", "spd"):
        raise ValueError(f"basis must be 'sp' or 'spd', got {basis!r}")
    rng = np.random.default_rng(seed)
    names = rng.choice(["H", "C", "N", "O"], size=num_atoms, p=[0.4, 0.2, 0.2, 0.2])
    Z = np.array([ELEMENTS[x] for x in names], dtype=np.float64)
    min_sep = 1.0 * ANGSTROM
    box = 1.6 * min_sep * max(1.0, num_atoms ** (1.0 / 3.0))
    pos = []
    while len(pos) < num_atoms:
        cand = rng.uniform(-box, box, 3)
        if all(np.linalg.norm(cand - p) >= min_sep for p in pos):
            pos.append(cand)
    pos = np.array(pos)
    shells = []
    for z, R in zip(Z, pos):
        ls = [0, 0] if z == 1 else [0, 0, 0, 1, 1]
        for l in ls:
            npr = int(rng.integers(1, 4))
            ex = np.exp(rng.uniform(math.log(0.1), math.log(50.0), npr))
            w = rng.uniform(0.2, 1.0, npr)
            co = w * np.array([_prim_norm(a, l) for a in ex])
            shells.append(Shell(center=R.copy(), l=l, exponents=ex, coefficients=co))
        if basis == "spd" and z != 1:
            ex = np.exp(rng.uniform(math.log(0.3), math.log(3.0), 1))
            shells.append(Shell(center=R.copy(), l=2, exponents=ex,
                                coefficients=np.array([_prim_norm(ex[0], 2)])))
    G = points_per_atom * num_atoms
    sig = 1.5
    which = rng.integers(0, num_atoms, G)
    coords = pos[which] + rng.normal(0.0, sig, (G, 3))
    d2 = ((coords[:, None, :] - pos[None, :, :]) ** 2).sum(-1)
    dens = np.exp(-0.5 * d2 / sig ** 2).mean(axis=1) / (2 * math.pi * sig ** 2) ** 1.5
    weights = rng.uniform(0.9, 1.1, G) / (G * dens)
    if grid == "becke":
        from .grids import Grids

        g = Grids(Molecule3D(charges=Z, positions=pos, shells=[], coords=coords,
                             weights=weights, nelectron=0))
        g.level = level
        g.build()
        coords = g.coords.cpu().numpy()
        weights = g.weights.cpu().numpy()
        G = weights.size
    elif grid != "cloud":
        raise ValueError(f"grid must be 'cloud' or 'becke', got {grid!r}")
    ne = int(Z.sum())
    ne -= ne % 2
    mol = Molecule3D(charges=Z, positions=pos, shells=shells, coords=coords, weights=weights,
                     nelectron=ne)
    e_nuc = 0.0
    for a in range(num_atoms):
        for b in range(a + 1, num_atoms):
            e_nuc += Z[a] * Z[b] / np.linalg.norm(pos[a] - pos[b])
    mol.energy_nuc = float(e_nuc)
    if with_integrals:
        ao, grad = ao_values(shells, coords, deriv=True)
        mol.ao = ao
        W = weights[:, None]
        mol.s1e = ao.T @ (W * ao)
        T = 0.5 * sum(grad[c].T @ (W * grad[c]) for c in range(3))
        vnuc = np.zeros(G)
        for z, R in zip(Z, pos):
            vnuc -= z / np.sqrt(((coords - R) ** 2).sum(-1) + 0.2)
        V = ao.T @ ((weights * vnuc)[:, None] * ao)
        mol.h1e = T + V
        n = ao.shape[1]
        naux = 3 * n
        fac = np.empty((naux, n, n))
        for p in range(naux):
            R = pos[rng.integers(0, num_atoms)]
            beta = math.exp(rng.uniform(math.log(0.2), math.log(2.0)))
            g = np.exp(-beta * ((coords - R) ** 2).sum(-1))
            fac[p] = 0.3 * (ao.T @ ((weights * g)[:, None] * ao))
        mol.eri_factors = fac
        if integrals == "analytic":
            analytic_integrals(mol)
        elif integrals != "model":
            raise ValueError(f"integrals must be 'model' or 'analytic', got {integrals!r}")
    return mol


def device_molecule(num_atoms: int, seed: int = 0, points_per_atom: int = 620,
                    basis: str = "sp"):
    """A synthetic molecule of the 3D configuration built on the GPU, for the
    sizes where the host model integrals are too slow (nao up to ~220, G up to
    2e5): geometry, shells and the Gaussian-cloud grid with positive random
    weights from ``synthetic_molecule``; AO values (``qex_td_eval_ao``), S,
    h1e = T + V_nuc (``qex_td_int1e``) and the density-fitted Coulomb factors
    (``qex_td_int3c2e`` / ``int2c2e`` / ``df_factors``) on the device.
    Returns (``graph.DeviceMolecule3D``, the host ``Molecule3D`` description)."""
    from . import integrals
    from .graph import DeviceMolecule3D
    from .numint import _dev, eval_ao

    import torch

    mol = synthetic_molecule(num_atoms, seed=seed, points_per_atom=points_per_atom,
                             with_integrals=False, basis=basis)
    ao = eval_ao(mol)
    S, T, V = integrals.int1e(mol)
    B = integrals.df_factors(mol)
    dev = DeviceMolecule3D(ao, _dev(np.asarray(mol.weights, np.float64), torch.float64), S, T + V,
                           B, int(mol.nelectron), float(mol.energy_nuc))
    return dev, mol
