"""Exchange-correlation functionals known to the GPU kernels.

The reference passes arbitrary JAX callables as ``xc_energy_density_fn``
(``qedft/train/od/scf.py:32-76``, wrapped by ``tree_util.Partial`` at
``qedft/train/od/train.py:102-105``).  A CUDA kernel cannot call back into
Python, so here the callable is one of the functionals below (or a
``Partial`` of one with its parameters); the SCF drivers read its kernel
description from it.  Each functional returns per-point values f(n):

  * amplitude-encoded convention (qedft): E_xc = dx * sum f, v_xc = dE_xc/dn;
  * local convention (jax_dft):          E_xc = dx * sum f n, v_xc = (dE_xc/dn)/dx.
"""

from __future__ import annotations

import ctypes
import functools

import numpy as np

from . import _native as N

EXPONENTIAL_COULOMB_AMPLITUDE = 1.071295
EXPONENTIAL_COULOMB_KAPPA = 1.0 / 2.385345


class XCFunctional:
    """Base class.  ``spec(params, convention)`` returns the native descriptor."""

    kind = N.QEX_XC_NONE

    def spec(self, params, convention: int):
        s = N.XcSpec()
        s.kind = self.kind
        s.convention = convention
        return s, None

    def __call__(self, density, params=None):
        raise TypeError(
            f"{type(self).__name__} is evaluated inside the SCF kernels; pass it as "
            "xc_energy_density_fn to the qex_gb300 SCF drivers")


class NoXC(XCFunctional):
    kind = N.QEX_XC_NONE


class PowerXC(XCFunctional):
    """f(n) = coefficient * (n + shift)^power.

    With coefficient=-0.73855, power=1/3 this is the exchange functional used by
    ``tests/test_scf_od.py:46-48`` (and with shift=1e-10 the regularised form of
    ``tests/test_scf_od.py:127-129``).
    """

    kind = N.QEX_XC_POWER

    def __init__(self, coefficient=-0.73855, power=1.0 / 3.0, shift=0.0):
        self.coefficient, self.power, self.shift = float(coefficient), float(power), float(shift)

    def spec(self, params, convention):
        s, keep = super().spec(params, convention)
        s.coefficient, s.power, s.shift = self.coefficient, self.power, self.shift
        return s, keep


class LDAExpCoulomb(XCFunctional):
    """Exponential-Coulomb uniform-gas LDA (jax_dft ``xc.get_lda_xc_energy_density_fn``,
    used at ``qedft/train/od/eval.py:79``).  Meant for the local convention."""

    kind = N.QEX_XC_LDA_EXP_COULOMB

    def __init__(self, amplitude=EXPONENTIAL_COULOMB_AMPLITUDE, kappa=EXPONENTIAL_COULOMB_KAPPA):
        self.amplitude, self.kappa = float(amplitude), float(kappa)

    def spec(self, params, convention):
        s, keep = super().spec(params, convention)
        s.lda_amplitude, s.lda_kappa = self.amplitude, self.kappa
        return s, keep


class WindowMLPFunctional(XCFunctional):
    """FP32 per-point MLP on a 17-point density window (two SiLU layers of 16).

    ``params`` is a list of three (W, b) pairs, W of shape (in, out), applied
    as x @ W + b (stax ``Dense``), as made by ``WindowMLP.build_network``.
    """

    kind = N.QEX_XC_WINDOW_MLP

    def __init__(self, normalization=2.0):
        self.normalization = float(normalization)

    @staticmethod
    def flatten(params) -> np.ndarray:
        (w1, b1), (w2, b2), (w3, b3) = params
        flat = np.concatenate([
            np.asarray(w1, np.float32).reshape(N.MLP_WINDOW * N.MLP_HIDDEN),
            np.asarray(b1, np.float32).reshape(N.MLP_HIDDEN),
            np.asarray(w2, np.float32).reshape(N.MLP_HIDDEN * N.MLP_HIDDEN),
            np.asarray(b2, np.float32).reshape(N.MLP_HIDDEN),
            np.asarray(w3, np.float32).reshape(N.MLP_HIDDEN),
            np.asarray(b3, np.float32).reshape(1),
        ])
        assert flat.size == N.MLP_NUM_PARAMS
        return np.ascontiguousarray(flat, dtype=np.float32)

    @staticmethod
    def unflatten(flat, dtype=np.float32):
        flat = np.asarray(flat, dtype)
        i = 0
        out = []
        for fi, fo in ((N.MLP_WINDOW, N.MLP_HIDDEN), (N.MLP_HIDDEN, N.MLP_HIDDEN), (N.MLP_HIDDEN, 1)):
            w = flat[i:i + fi * fo].reshape(fi, fo)
            i += fi * fo
            b = flat[i:i + fo]
            i += fo
            out.append((w, b))
        return out

    def spec(self, params, convention):
        if params is None:
            raise ValueError("WindowMLPFunctional needs params")
        s, _ = super().spec(params, convention)
        flat = self.flatten(params)
        s.normalization = self.normalization
        s.mlp_params_host = flat.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        return s, flat  # keep the host buffer alive for the call


class Partial:
    """Minimal stand-in for ``jax.tree_util.Partial``: a functional with bound
    keyword arguments (``params``), as built at ``qedft/train/od/train.py:102-105``."""

    def __init__(self, func, *args, **kwargs):
        self.func, self.args, self.kwargs = func, args, kwargs

    def __call__(self, *args, **kwargs):
        return self.func(*self.args, *args, **{**self.kwargs, **kwargs})


def resolve(xc):
    """Return (XCFunctional, params) from a functional, a Partial, a
    functools.partial or an ``xc_energy_density_fn`` built by
    ``qex_gb300.networks.build_xc_functional``."""
    params = None
    obj = xc
    for _ in range(8):
        if isinstance(obj, XCFunctional):
            return obj, params
        if isinstance(obj, (Partial, functools.partial)):
            kw = obj.kwargs if isinstance(obj, Partial) else obj.keywords
            if "params" in kw:
                params = kw["params"]
            obj = obj.func
            continue
        inner = getattr(obj, "functional", None)
        if isinstance(inner, XCFunctional):
            return inner, params
        break
    raise TypeError(
        "xc_energy_density_fn must be a qex_gb300 XC functional (PowerXC, LDAExpCoulomb, "
        "WindowMLPFunctional), a Partial of one, or built by qex_gb300.networks; arbitrary "
        f"Python callables cannot run inside the CUDA kernels (got {type(xc).__name__})")
