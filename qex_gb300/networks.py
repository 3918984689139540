"""Network plug-in API mirroring ``qedft/models/networks.py`` and
``qedft/models/wrappers.py``.

``KohnShamNetwork.build_network(grids) -> (init_fn, apply_fn)`` with
``init_fn(rng, input_shape) -> (output_shape, params)`` and
``apply_fn(params, inputs)`` (``qedft/models/networks.py:43-75``), and
``build_xc_functional(network, grids, config) -> (init_fn(rng) -> params,
xc_energy_density_fn(density, params))`` with the reversed argument order of
``qedft/models/wrappers.py:267-299``.  The ``xc_energy_density_fn`` returned
here carries its GPU kernel description, so it can be passed (bound to its
params with ``Partial``) to the SCF drivers of ``qex_gb300.od``.
"""

from __future__ import annotations

from typing import Protocol

import numpy as np

from . import _native as N
from .xc import LDAExpCoulomb, WindowMLPFunctional, XCFunctional


class KohnShamNetwork(Protocol):
    def build_network(self, grids):  # pragma: no cover - protocol
        raise NotImplementedError


def _rng(rng):
    if isinstance(rng, np.random.Generator):
        return rng
    return np.random.default_rng(int(rng))


def glorot_uniform(rng, fan_in, fan_out, dtype=np.float32):
    lim = np.sqrt(6.0 / (fan_in + fan_out))
    return rng.uniform(-lim, lim, size=(fan_in, fan_out)).astype(dtype)


class WindowMLP:
    """Local XC network: eps_i = MLP(n[i-8..i+8] / norm), 17 -> 16 -> 16 -> 1, SiLU.

    The per-point MLP of ``qedft/models/classical/classical_models.py:123-174``
    (input divided by ``density_normalization_factor``) with a zero-padded
    17-point window as input; Glorot-uniform weights, zero biases.
    """

    def __init__(self, config_dict: dict | None = None):
        self.config = {"network_type": "mlp", "n_neurons": N.MLP_HIDDEN, "n_layers": 2,
                       "activation": "silu", "window": N.MLP_WINDOW,
                       "density_normalization_factor": 2.0}
        if config_dict:
            self.config.update(config_dict)
        if (self.config["n_neurons"] != N.MLP_HIDDEN or self.config["n_layers"] != 2
                or self.config["window"] != N.MLP_WINDOW or self.config["activation"] != "silu"):
            raise ValueError("the GPU window MLP is fixed at window 17, two SiLU layers of 16")
        self.functional = WindowMLPFunctional(self.config["density_normalization_factor"])

    def build_network(self, grids):
        del grids
        functional = self.functional

        def init_fn(rng, input_shape=None):
            del input_shape
            g = _rng(rng)
            params = [
                (glorot_uniform(g, N.MLP_WINDOW, N.MLP_HIDDEN), np.zeros(N.MLP_HIDDEN, np.float32)),
                (glorot_uniform(g, N.MLP_HIDDEN, N.MLP_HIDDEN), np.zeros(N.MLP_HIDDEN, np.float32)),
                (glorot_uniform(g, N.MLP_HIDDEN, 1), np.zeros(1, np.float32)),
            ]
            return (-1, 1), params

        def apply_fn(params, inputs, **kwargs):
            return functional(inputs, params)

        apply_fn.functional = functional
        return init_fn, apply_fn


class LDA:
    """The exponential-Coulomb LDA as a (parameter-free) network."""

    def __init__(self, config_dict: dict | None = None):
        self.config = {"network_type": "lda"}
        if config_dict:
            self.config.update(config_dict)
        self.functional = LDAExpCoulomb()

    def build_network(self, grids):
        functional = self.functional

        def init_fn(rng, input_shape=None):
            return (-1,), None

        def apply_fn(params, inputs, **kwargs):
            return functional(inputs, params)

        apply_fn.functional = functional
        return init_fn, apply_fn


class _XCEnergyDensityFn:
    """``xc_energy_density_fn(density, params)`` carrying its kernel functional."""

    def __init__(self, functional: XCFunctional):
        self.functional = functional

    def __call__(self, density, params=None, **kwargs):
        return self.functional(density, params)


def build_xc_functional(network, grids, config: dict | None = None):
    """(init_fn(rng) -> params, xc_energy_density_fn(density, params)).

    Mirrors ``qedft/models/wrappers.py:267-299``.  The self-interaction and
    negativity wrappers of ``wrap_network`` are not part of the GPU path.
    """
    config = dict(config or {})
    if config.get("wrap_self_interaction") or config.get("wrap_with_negative_transform"):
        raise NotImplementedError("self-interaction / negativity wrappers are not on the GPU path")
    net_init, net_apply = network
    functional = getattr(net_apply, "functional", None)
    if not isinstance(functional, XCFunctional):
        raise TypeError("network apply_fn does not carry a qex_gb300 XC functional")

    def init_fn(rng, **kwargs):
        _, params = net_init(rng, input_shape=(-1, np.asarray(grids).shape[0], 1))
        return params

    return init_fn, _XCEnergyDensityFn(functional)
