"""1D Kohn-Sham SCF on GB300: the drop-in for ``qedft.train.od``."""

from . import engine, jit_scf, scf, utils  # noqa: F401
from .engine import Ks1dEngine, Molecule1D, PackedBatch, SolveConfig  # noqa: F401
