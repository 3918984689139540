"""Seeded synthetic 1D workloads with the shapes of the benchmark configurations.

* ``batched_molecules``: 1-4 nuclei of charge 1-3 at positions uniform in
  [-3, 3] bohr, neutral, grids of 257 / 385 / 513 points at spacing 0.08 bohr
  centred at 0 (the batched configuration, 4096 molecules).
* ``h2_config``: two unit charges at +-0.7 bohr, 2 electrons, 513 points
  (the plain single-solve configuration).
"""

from __future__ import annotations

import numpy as np

from .engine import Molecule1D


def batched_molecules(count: int, seed: int = 0, grid_choices=(257, 385, 513), spacing=0.08,
                      max_nuclei=4, max_charge=3, extent=3.0):
    rng = np.random.default_rng(seed)
    mols = []
    for _ in range(count):
        n = int(rng.choice(grid_choices))
        m = int(rng.integers(1, max_nuclei + 1))
        z = rng.integers(1, max_charge + 1, m).astype(np.float64)
        r = rng.uniform(-extent, extent, m)
        mols.append(Molecule1D(num_grids=n, grid_spacing=spacing, locations=r, nuclear_charges=z,
                               num_electrons=int(z.sum())))
    return mols


def h2_config(separation=1.4, num_grids=513, spacing=0.08):
    h = 0.5 * separation
    return Molecule1D(num_grids=num_grids, grid_spacing=spacing, locations=[-h, h],
                      nuclear_charges=[1.0, 1.0], num_electrons=2)
