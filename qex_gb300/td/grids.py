"""Molecular integration grids (pyscf ``dft.gen_grid.Grids`` as the reference
builds them: ``qedft/data_io/td/dataset_generation.py:139-142``,
``qedft/train/td/rks_legacy.py:46``).

Atom-centred grids: the Treutler-Ahlrichs M4 radial mapping on Chebyshev
nodes of the second kind (Treutler, Ahlrichs, J. Chem. Phys. 102, 346 (1995)),
an angular product rule (Gauss-Legendre in cos(theta) x uniform phi; the
Lebedev tables pyscf uses are not in this image), and Becke's fuzzy-cell
partition with his atomic-size adjustment from Bragg-Slater radii and
Stratmann's switching function (or Becke's).  The partition, O(points x
atoms^2), runs on the GPU (``qex_td_becke_grid``); the radial and angular
tables are built on the host.
"""

from __future__ import annotations

import math

import numpy as np

from .. import _native as N
from . import _lib

ANGSTROM = 1.0 / 0.52917721092
# Bragg-Slater radii (Angstrom), with Becke's 0.35 for hydrogen
BRAGG_RADII = {1: 0.35, 2: 1.40, 3: 1.45, 4: 1.05, 5: 0.85, 6: 0.70, 7: 0.65, 8: 0.60, 9: 0.50,
               10: 1.50}
# Treutler-Ahlrichs radial scaling xi
TREUTLER_XI = {1: 0.8, 2: 0.9, 3: 1.8, 4: 1.4, 5: 1.3, 6: 1.1, 7: 0.9, 8: 0.9, 9: 0.9, 10: 0.9}
# radial nodes per level for the first and second rows, angular theta nodes per level
RADIAL = ((10, 30, 40, 50, 60, 70, 80, 90, 100, 200), (15, 40, 60, 75, 90, 105, 120, 135, 150, 200))
ANGULAR_THETA = (6, 8, 10, 12, 14, 16, 18, 20, 22, 24)


def stratmann(g):
    """Stratmann, Scuseria, Frisch's switching polynomial (a = 0.64)."""
    a = 0.64
    g = np.asarray(g, dtype=np.float64)
    m = g / a
    m2 = m * m
    out = (1.0 / 16.0) * (m * (35.0 + m2 * (-35.0 + m2 * (21.0 - 5.0 * m2))))
    return np.where(g <= -a, -1.0, np.where(g >= a, 1.0, out))


def original_becke(g):
    """Becke's switching function: three iterations of 1.5 g - 0.5 g^3."""
    g = np.asarray(g, dtype=np.float64)
    for _ in range(3):
        g = (3.0 - g * g) * g * 0.5
    return g


def treutler_ahlrichs(n, xi=1.0):
    """M4 radial nodes r and weights r^2 dr (ascending r)."""
    i = np.arange(1, n + 1)
    step = math.pi / (n + 1)
    x = np.cos(i * step)
    ln2 = 1.0 / math.log(2.0)
    r = -ln2 * (1.0 + x) ** 0.6 * np.log((1.0 - x) / 2.0)
    dr = step * np.sin(i * step) * ln2 * (1.0 + x) ** 0.6 * (
        -0.6 / (1.0 + x) * np.log((1.0 - x) / 2.0) + 1.0 / (1.0 - x))
    r, dr = xi * r[::-1], xi * dr[::-1]
    return r, r * r * dr


def angular_product(n_theta):
    """Unit vectors and weights (summing to 4 pi) of the product rule with
    n_theta Gauss-Legendre nodes in cos(theta) and 2 n_theta uniform phi."""
    t, wt = np.polynomial.legendre.leggauss(n_theta)
    n_phi = 2 * n_theta
    phi = (np.arange(n_phi) + 0.5) * (2.0 * math.pi / n_phi)
    st = np.sqrt(1.0 - t * t)
    u = np.stack([np.outer(st, np.cos(phi)).ravel(), np.outer(st, np.sin(phi)).ravel(),
                  np.repeat(t, n_phi)], axis=1)
    w = np.repeat(wt, n_phi) * (2.0 * math.pi / n_phi)
    return u, w


def becke_size_adjust(charges):
    """Becke's a_bc from the ratio of Bragg-Slater radii (clipped to |a| <= 1/2)."""
    R = np.array([BRAGG_RADII.get(int(z), 1.0) for z in charges])
    chi = R[:, None] / R[None, :]
    u = (chi - 1.0) / (chi + 1.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(np.abs(u) > 0.0, u / (u * u - 1.0), 0.0)
    return np.clip(a, -0.5, 0.5)


def radial_for(z, level):
    row = 0 if int(z) <= 2 else 1
    return RADIAL[row][level]


def grid_tables(charges, level=3):
    """Per-atom radial tables and the angular rule for ``level`` (0-9)."""
    rad = [treutler_ahlrichs(radial_for(z, level), TREUTLER_XI.get(int(z), 1.0))
           for z in charges]
    u, w = angular_product(ANGULAR_THETA[level])
    return rad, u, w


class Grids:
    """``gen_grid.Grids(mol)``: set ``level`` and ``becke_scheme`` (``stratmann``
    or ``original_becke``), then ``build()`` fills ``coords`` (G, 3) and
    ``weights`` (G) as device tensors.  ``mol`` needs ``charges`` and
    ``positions`` (bohr)."""

    def __init__(self, mol):
        self.mol = mol
        self.level = 3
        self.becke_scheme = stratmann
        self.radii_adjust = True
        self.coords = None
        self.weights = None

    def build(self):
        torch = N.require_cuda()
        charges = np.asarray(self.mol.charges)
        xyz = np.ascontiguousarray(self.mol.positions, dtype=np.float64).reshape(-1, 3)
        natom = xyz.shape[0]
        rad, u, w = grid_tables(charges, int(self.level))
        nrad = np.array([r.size for r, _ in rad], dtype=np.int32)
        roff = np.concatenate([[0], np.cumsum(nrad)[:-1]]).astype(np.int64)
        off = np.concatenate([[0], np.cumsum(nrad.astype(np.int64) * u.shape[0])]).astype(np.int64)
        G = int(off[-1])
        scheme = 1 if self.becke_scheme is stratmann or self.becke_scheme == "stratmann" else 0
        dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
        t = {"xyz": dev(xyz), "off": dev(off), "nrad": dev(nrad), "roff": dev(roff),
             "r": dev(np.concatenate([r for r, _ in rad])),
             "w": dev(np.concatenate([wr for _, wr in rad])),
             "u": dev(u), "uw": dev(w)}
        adj = dev(becke_size_adjust(charges)) if self.radii_adjust else None
        coords = torch.empty((G, 3), dtype=torch.float64, device="cuda")
        weights = torch.empty(G, dtype=torch.float64, device="cuda")
        N.check(_lib.lib().qex_td_becke_grid(
            natom, _lib.p(t["xyz"]), _lib.p(adj) if adj is not None else None, _lib.p(t["off"]),
            _lib.p(t["nrad"]), _lib.p(t["roff"]), _lib.p(t["r"]), _lib.p(t["w"]), u.shape[0],
            _lib.p(t["u"]), _lib.p(t["uw"]), scheme, G, _lib.p(coords), _lib.p(weights),
            _lib.stream()), "qex_td_becke_grid")
        self.coords, self.weights = coords, weights
        return self
