"""qex_gb300: GB300-native (sm_103a) Kohn-Sham SCF hot path of pasqal-io/qex.

The compute path is the CUDA library ``qex_gb300/lib/libqex_gb300.so`` (C ABI
in ``include/``); Python mirrors the reference's interfaces on top of it.
"""

from . import networks, xc  # noqa: F401
from .xc import KSRFunctional, LDAExpCoulomb, Partial, PowerXC, WindowMLPFunctional  # noqa: F401

__version__ = "0.1.0"
