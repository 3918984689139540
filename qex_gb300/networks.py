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
from .xc import LDAExpCoulomb, NeuralMLPFunctional, Partial, WindowMLPFunctional, XCFunctional


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


def glorot_normal(rng, fan_in, fan_out, dtype=np.float32):
    """jax.nn.initializers.glorot_normal (stax ``Dense``'s default): a normal
    truncated at two standard deviations, variance 2 / (fan_in + fan_out)."""
    std = np.sqrt(2.0 / (fan_in + fan_out)) / 0.87962566103423978
    w = rng.normal(0.0, std, size=(fan_in, fan_out))
    bad = np.abs(w) > 2.0 * std
    while bad.any():
        w[bad] = rng.normal(0.0, std, size=int(bad.sum()))
        bad = np.abs(w) > 2.0 * std
    return w.astype(dtype)


def dense_stack_params(rng, fan_in, n_neurons, n_layers, n_outputs=1):
    """stax.serial([Dense(n_neurons), activation] x n_layers, Dense(n_outputs))
    parameters (``qedft/models/classical/classical_models.py:77-115``):
    (W, b) per Dense layer (Glorot-normal W, normal(1e-6) b), () per activation."""
    g = _rng(rng)
    params = []
    fin = fan_in
    for _ in range(n_layers):
        params.append((glorot_normal(g, fin, n_neurons),
                       (g.normal(0.0, 1e-6, n_neurons)).astype(np.float32)))
        params.append(())
        fin = n_neurons
    params.append((glorot_normal(g, fin, n_outputs), (g.normal(0.0, 1e-6, n_outputs)).astype(np.float32)))
    return params


class _DenseNetwork:
    """(init_fn, apply_fn) of a bare dense stack; apply_fn evaluates it on the
    GPU (no wrappers).  ``template`` is the unwrapped functional."""

    def __init__(self, template: NeuralMLPFunctional, fan_in):
        self.template, self.fan_in = template, int(fan_in)

    def init_fn(self, rng, input_shape=None):
        params = dense_stack_params(rng, self.fan_in, self.template.n_neurons,
                                    self.template.n_layers)
        out = (input_shape[:-1] + (1,)) if input_shape and self.template.local else (1,)
        return out, params

    def apply_fn(self, params, inputs, **kwargs):
        from .od.xc_eval import xc_energy_and_potential

        n = np.asarray(inputs, dtype=np.float64).reshape(-1)
        t = self.template
        bare = NeuralMLPFunctional(t.local, t.n_neurons, t.n_layers, t.activation,
                                   t.normalization, False, False, n.size)
        _, _, vals = xc_energy_and_potential(n, Partial(bare, params=params),
                                             np.arange(n.size) * 1.0, "amplitude")
        return vals if t.local else np.array([vals.sum()])

    def __iter__(self):
        return iter((self.init_fn, self.apply_fn))


class LocalMLP:
    """``qedft/models/networks.py:83-109``: the dense network applied at every
    grid point to n_i / density_normalization_factor
    (``build_local_mlp``, ``qedft/models/classical/classical_models.py:123-174``).
    Default config: n_neurons 64, n_layers 3, tanh, normalization 2.0, wrapped
    with the negativity transform (``wrap_with_negative_transform``)."""

    def __init__(self, config_dict: dict | None = None):
        self.config = {"network_type": "mlp", "wrap_self_interaction": False,
                       "wrap_with_negative_transform": True, "use_amplitude_encoding": False}
        if config_dict is not None:
            self.config.update(config_dict)
        if self.config.get("use_amplitude_encoding") is True:
            raise ValueError("Set use_amplitude_encoding to False.")

    def build_network(self, grids):
        if grids is None:
            raise ValueError("grids must be provided for local MLP")
        t = NeuralMLPFunctional(True, self.config.get("n_neurons", 64),
                                self.config.get("n_layers", 3),
                                self.config.get("activation", "tanh"),
                                self.config.get("density_normalization_factor", 2.0),
                                False, False, 1)
        return _DenseNetwork(t, 1)


class GlobalMLP:
    """``qedft/models/networks.py:112-138``: the dense network on the whole
    density vector / density_normalization_factor, one scalar out
    (``build_global_mlp``, ``classical_models.py:177-224``).  Default config:
    network_type "mlp_ksr" (amplitude encoding), n_neurons 64, n_layers 3,
    tanh, normalization 2.0, wrapped with the self-interaction layer and the
    negativity transform."""

    def __init__(self, config_dict: dict | None = None):
        self.config = {"network_type": "mlp_ksr", "wrap_self_interaction": True,
                       "wrap_with_negative_transform": True, "use_amplitude_encoding": True}
        if config_dict is not None:
            self.config.update(config_dict)
        if self.config.get("use_amplitude_encoding") is False:
            raise ValueError("Set use_amplitude_encoding to True.")

    def build_network(self, grids):
        if grids is None:
            raise ValueError("grids must be provided for global MLP")
        n = int(np.asarray(grids).shape[0])
        t = NeuralMLPFunctional(False, self.config.get("n_neurons", 64),
                                self.config.get("n_layers", 3),
                                self.config.get("activation", "tanh"),
                                self.config.get("density_normalization_factor", 2.0),
                                False, False, n)
        return _DenseNetwork(t, n)


# network types whose functional is global (amplitude encoded), qedft/models/wrappers.py:170-178
_GLOBAL_TYPES = ("gadqc", "gadqc_with_mlp", "conv_dqc", "conv_adqc", "mlp_ksr", "conv_dqc_tfm",
                 "conv_adqc_tfm")


def _wrap_dense(network: _DenseNetwork, grids, config):
    """``wrap_network`` (``qedft/models/wrappers.py:162-217``) for the dense
    networks: self-interaction, then negativity, then (global types) the mean."""
    t = network.template
    is_global = config.get("network_type") in _GLOBAL_TYPES
    if is_global == t.local:
        raise ValueError(f"network_type {config.get('network_type')!r} does not match a "
                         f"{'local' if t.local else 'global'} network")
    si = bool(config.get("wrap_self_interaction", False))
    neg = bool(config.get("wrap_with_negative_transform", False))
    functional = NeuralMLPFunctional(t.local, t.n_neurons, t.n_layers, t.activation,
                                     t.normalization, si, neg, t.num_inputs)
    n = int(np.asarray(grids).shape[0])

    def init_fn(rng, **kwargs):
        # the local network is initialised with input_shape (-1, N, 1), the
        # global one with (1,) (wrappers.py:62-75); the Dense shapes follow the fan-in
        _, params = network.init_fn(rng, (-1, n, 1) if t.local else (1,))
        if si:
            params = [(), ((), params), (np.array(1.0, np.float32),)]
        if neg:
            params = [params, ()]
        return params

    return init_fn, _XCEnergyDensityFn(functional)


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

    Mirrors ``qedft/models/wrappers.py:267-299``.  For the dense networks
    (``LocalMLP``, ``GlobalMLP``) the config's ``wrap_self_interaction`` and
    ``wrap_with_negative_transform`` wrappers and the global mean are part of
    the GPU functional; the fixed-shape window MLP and the LDA take none.
    """
    config = dict(config or {})
    if isinstance(network, tuple) and isinstance(getattr(network[1], "__self__", None),
                                                 _DenseNetwork):
        network = network[1].__self__  # (init_fn, apply_fn) unpacked from build_network
    if isinstance(network, _DenseNetwork):
        return _wrap_dense(network, grids, config)
    if config.get("wrap_self_interaction") or config.get("wrap_with_negative_transform"):
        raise NotImplementedError("the self-interaction / negativity wrappers apply to the dense "
                                  "networks (LocalMLP, GlobalMLP) and the KSR model")
    net_init, net_apply = network
    functional = getattr(net_apply, "functional", None)
    if not isinstance(functional, XCFunctional):
        raise TypeError("network apply_fn does not carry a qex_gb300 XC functional")

    def init_fn(rng, **kwargs):
        _, params = net_init(rng, input_shape=(-1, np.asarray(grids).shape[0], 1))
        return params

    return init_fn, _XCEnergyDensityFn(functional)


# ---------------------------------------------------------------------------
# Global-local convolutional KSR functional
# ---------------------------------------------------------------------------

KSR_DEFAULT_CONFIG = {
    "num_global_filters": 16,
    "num_local_filters": 16,
    "num_local_conv_layers": 2,
    "activation": "swish",
    "minval": 0.1,
    "maxval": 2.385345,
    "downsample_factor": 0,
}


def _is_power_of_two(n: int) -> bool:
    return n > 0 and (n & (n - 1)) == 0


class KSRNetwork:
    """(init_fn, apply_fn) pair of the global-local conv network, as built by
    jax_dft ``neural_xc.build_global_local_conv_net`` (called at
    ``qedft/models/classical/global_ksr_model.py:62-71``).  Carries the GPU
    description; ``self_interaction`` is set by
    ``wrap_network_with_self_interaction_layer``."""

    def __init__(self, channels, grids, minval, maxval, self_interaction=False):
        self.channels = int(channels)
        self.grids = np.asarray(grids, dtype=np.float64)
        self.minval, self.maxval = float(minval), float(maxval)
        self.self_interaction = bool(self_interaction)

    def _init_net(self, g):
        c = self.channels
        # eta ~ normal(0, 0.01) (the exponential convolution's initialiser);
        # bias-free conv kernels Glorot-normal over (width * channels) fans
        eta = g.normal(0.0, 0.01, size=c - 1)
        std3 = np.sqrt(2.0 / (3 * c + 3 * c))
        std1 = np.sqrt(2.0 / (c + 1))
        w1 = np.clip(g.normal(0.0, std3, size=(3, c, c)), -2 * std3, 2 * std3)
        w2 = np.clip(g.normal(0.0, std3, size=(3, c, c)), -2 * std3, 2 * std3)
        w3 = np.clip(g.normal(0.0, std1, size=(1, c, 1)), -2 * std1, 2 * std1)
        block = [(), ((), [(eta,)]), ()]
        return [block, (w1,), (), (w2,), (), (w3,), ()]

    def init_fn(self, rng, input_shape=None):
        g = _rng(rng)
        net = self._init_net(g)
        if self.self_interaction:
            return input_shape, [(), ((), net), (np.array(1.0),)]
        return input_shape, net

    def __iter__(self):
        return iter((self.init_fn, self.apply_fn))

    def apply_fn(self, params, inputs, **kwargs):
        raise NotImplementedError(
            "the KSR network is evaluated by its global functional on the GPU; use "
            "global_functional(network, grids)")


def build_global_local_conv_net(num_global_filters, num_local_filters, num_local_conv_layers,
                                activation, grids, minval, maxval, downsample_factor):
    """jax_dft ``neural_xc.build_global_local_conv_net`` with the arguments of
    ``qedft/models/classical/global_ksr_model.py:62-71``.  The GPU kernels take
    equal global and local filter counts of 8 or 16, two local layers, swish
    and no downsampling; the grid must have 2^k + 1 points (ValueError
    otherwise, as ``tests/test_global_ksr_model.py:103-111`` expects)."""
    n = int(np.asarray(grids).shape[0])
    if not _is_power_of_two(n - 1):
        raise ValueError(f"the number of grid points must be 2^k + 1, got {n}")
    if num_global_filters != num_local_filters or num_global_filters not in (8, 16):
        raise ValueError("the GPU KSR network takes 8 or 16 global and local filters")
    if num_local_conv_layers != 2 or activation != "swish" or downsample_factor != 0:
        raise ValueError("the GPU KSR network has two swish local layers and no downsampling")
    return KSRNetwork(num_global_filters, grids, minval, maxval)


def wrap_network_with_self_interaction_layer(network, grids, interaction_fn=None):
    """jax_dft ``neural_xc.wrap_network_with_self_interaction_layer``
    (``global_ksr_model.py:73-77``); the self-interaction Hartree term uses the
    exponential Coulomb interaction with its default constants."""
    if not isinstance(network, KSRNetwork):
        raise TypeError("expected a network from build_global_local_conv_net")
    return KSRNetwork(network.channels, grids, network.minval, network.maxval,
                      self_interaction=True)


def global_functional(network, grids):
    """jax_dft ``neural_xc.global_functional`` (``global_ksr_model.py:79``):
    (init_fn(rng) -> params, xc_energy_density_fn(density, params) -> eps).

    ``xc_energy_density_fn`` evaluates the network on the GPU
    (``qex_ksr1d_eval``) and carries its ``KSRFunctional``, so it can be
    passed (bound with ``Partial``) to the SCF drivers of ``qex_gb300.od``."""
    from .xc import KSRFunctional

    if not isinstance(network, KSRNetwork) or not network.self_interaction:
        raise NotImplementedError(
            "the GPU KSR functional includes the self-interaction layer; wrap the network "
            "with wrap_network_with_self_interaction_layer first")
    grids = np.asarray(grids, dtype=np.float64)
    functional = KSRFunctional(network.channels, network.minval, network.maxval)

    def init_fn(rng):
        return network.init_fn(rng, (-1, grids.shape[0], 1))[1]

    def xc_energy_density_fn(density, params):
        from .od import utils as _u
        from .od.xc_eval import ksr_eval

        n = np.asarray(density, dtype=np.float64)
        if n.shape != grids.shape:
            raise ValueError(f"density must have shape {grids.shape}, got {n.shape}")
        return ksr_eval([n], _u.get_dx(grids), Partial(functional, params=params),
                        potential=False)[0][2]

    xc_energy_density_fn.functional = functional
    return init_fn, xc_energy_density_fn


def create_ksr_model_from_config(grids, config: dict | None = None):
    """(network, init_fn, apply_fn) as ``qedft/models/classical/global_ksr_model.py:32-80``."""
    cfg = dict(KSR_DEFAULT_CONFIG)
    if config is not None:
        cfg = {k: config.get(k, v) for k, v in KSR_DEFAULT_CONFIG.items()}
    network = build_global_local_conv_net(
        num_global_filters=cfg["num_global_filters"], num_local_filters=cfg["num_local_filters"],
        num_local_conv_layers=cfg["num_local_conv_layers"], activation=cfg["activation"],
        grids=grids, minval=cfg["minval"], maxval=cfg["maxval"],
        downsample_factor=cfg["downsample_factor"])
    network = wrap_network_with_self_interaction_layer(network, grids=grids)
    init_fn, apply_fn = global_functional(network, grids=grids)
    return network, init_fn, apply_fn


def ksr_params_dict(params) -> dict:
    """Plain-array form of a KSR parameter tree: eta, conv (two kernels), out, width."""
    from .xc import KSRFunctional

    return KSRFunctional.as_dict(params)
