"""Grid and interaction helpers with the jax_dft ``utils`` names used by qedft.

``exponential_coulomb`` and ``soft_coulomb`` are interaction descriptors: they
can be called on host arrays like the jax_dft functions (for inspection), and
the SCF drivers read their kernel parameters from them.
"""

from __future__ import annotations

import numpy as np

from .. import _native as N

EXPONENTIAL_COULOMB_AMPLITUDE = 1.071295
EXPONENTIAL_COULOMB_KAPPA = 1.0 / 2.385345


def get_dx(grids) -> float:
    """(max - min) / (N - 1), jax_dft ``utils.get_dx`` (``qedft/train/od/scf.py:50``)."""
    grids = np.asarray(grids)
    if grids.ndim != 1:
        raise ValueError("grids must be one-dimensional")
    return float((grids.max() - grids.min()) / (grids.size - 1))


class _Interaction:
    def __init__(self, kind, a, b, name):
        self.kind, self.a, self.b, self.__name__ = kind, float(a), float(b), name

    def __call__(self, displacements):
        d = np.asarray(displacements, dtype=np.float64)
        if self.kind == N.QEX_INTERACTION_EXPONENTIAL:
            return self.a * np.exp(-np.abs(d) * self.b)
        return 1.0 / np.sqrt(d * d + self.a)

    def __repr__(self):
        return f"<interaction {self.__name__}>"


exponential_coulomb = _Interaction(N.QEX_INTERACTION_EXPONENTIAL, EXPONENTIAL_COULOMB_AMPLITUDE,
                                   EXPONENTIAL_COULOMB_KAPPA, "exponential_coulomb")
soft_coulomb = _Interaction(N.QEX_INTERACTION_SOFT_COULOMB, 1.0, 0.0, "soft_coulomb")


def make_exponential_coulomb(amplitude=EXPONENTIAL_COULOMB_AMPLITUDE, kappa=EXPONENTIAL_COULOMB_KAPPA):
    return _Interaction(N.QEX_INTERACTION_EXPONENTIAL, amplitude, kappa, "exponential_coulomb")


def make_soft_coulomb(soften_factor=1.0):
    return _Interaction(N.QEX_INTERACTION_SOFT_COULOMB, soften_factor, 0.0, "soft_coulomb")


def interaction_descriptor(fn):
    if isinstance(fn, _Interaction):
        return fn.kind, fn.a, fn.b
    raise TypeError("interaction_fn must be qex_gb300.od.utils.exponential_coulomb or soft_coulomb "
                    "(or made by make_exponential_coulomb / make_soft_coulomb)")


def gaussian(grids, center, sigma=1.0):
    """Normalised Gaussian (jax_dft ``utils.gaussian``)."""
    grids = np.asarray(grids, dtype=np.float64)
    return np.exp(-0.5 * ((grids - center) / sigma) ** 2) / (np.sqrt(2.0 * np.pi) * sigma)
