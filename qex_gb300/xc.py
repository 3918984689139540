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

    def __init__(self, normalization=2.0, precision="fp32"):
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision is 'fp32' (the configuration's network) or 'fp64' "
                             "(a checking mode)")
        self.normalization = float(normalization)
        self.precision = precision
        self._dev = None

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
        if self.precision == "fp64":
            # the parameters in FP64 as given (not rounded to FP32): the network
            # then runs in FP64 in the SCF and in the adjoint step
            torch = N.require_cuda()
            flat64 = self.flatten64(params)
            key = flat64.tobytes()
            if self._dev is None or self._dev[0] != key:
                self._dev = (key, torch.as_tensor(flat64, device="cuda"))
            s.mlp_params64 = self._dev[1].data_ptr()
            return s, (flat, self._dev[1])
        return s, flat  # keep the host buffer alive for the call

    @staticmethod
    def flatten64(params) -> np.ndarray:
        (w1, b1), (w2, b2), (w3, b3) = params
        flat = np.concatenate([np.asarray(a, np.float64).reshape(-1)
                               for a in (w1, b1, w2, b2, w3, b3)])
        assert flat.size == N.MLP_NUM_PARAMS
        return np.ascontiguousarray(flat)


class KSRFunctional(XCFunctional):
    """Global-local convolutional KSR network with the self-interaction layer
    (``qedft/models/classical/global_ksr_model.py:32-80``), FP32 on the GPU.

    A whole-grid functional: eps_i depends on the density at every point
    (through the exponential global convolutions and the self-interaction
    Hartree term), so the kernels evaluate it per molecule and back-propagate
    the cotangent through it for v_xc.  ``params`` is the stax parameter tree
    of ``create_ksr_model_from_config`` (the nesting of the trained
    ``data/od/h2/h2_optimal.pkl``) or the dict form of
    ``qex_gb300.networks.ksr_params_dict``.
    """

    kind = N.QEX_XC_KSR

    def __init__(self, channels=N.KSR_CHANNELS, minval=0.1, maxval=2.385345):
        if channels not in (8, 16):
            raise ValueError("the GPU KSR network has 8 or 16 channels")
        self.channels = int(channels)
        self.minval, self.maxval = float(minval), float(maxval)
        self._dev = None  # (packed bytes, device buffer)

    @staticmethod
    def as_dict(params) -> dict:
        if isinstance(params, dict):
            return params
        net = params[1][1]
        return {"eta": np.asarray(net[0][1][1][0][0]),
                "conv": [np.asarray(layer[0]) for layer in net[1:-2] if len(layer) == 1],
                "out": np.asarray(net[-2][0]), "width": float(np.asarray(params[2][0]))}

    def pack(self, params) -> np.ndarray:
        p = self.as_dict(params)
        c = self.channels
        w1, w2 = (np.asarray(w, np.float32) for w in p["conv"])
        w3 = np.asarray(p["out"], np.float32)
        eta = np.asarray(p["eta"], np.float32).reshape(-1)
        if w1.shape != (3, c, c) or w2.shape != (3, c, c) or w3.shape != (1, c, 1) or eta.size != c - 1:
            raise ValueError(f"KSR params do not match {c} channels")
        flat = np.concatenate([w1.reshape(-1), w2.reshape(-1), w3.reshape(-1), eta,
                               np.asarray([p["width"]], np.float32)])
        assert flat.size == N.ksr_num_params(c)
        return np.ascontiguousarray(flat, dtype=np.float32)

    def device_params(self, params):
        """The packed network on the current CUDA device (re-uploaded only when it changes)."""
        torch = N.require_cuda()
        flat = self.pack(params)
        key = flat.tobytes()
        if self._dev is None or self._dev[0] != key or self._dev[1].device != torch.device(
                "cuda", torch.cuda.current_device()):
            self._dev = (key, torch.as_tensor(flat, device="cuda"))
        return self._dev[1]

    def spec(self, params, convention):
        if params is None:
            raise ValueError("KSRFunctional needs params")
        s, _ = super().spec(params, convention)
        buf = self.device_params(params)
        s.ksr_params = buf.data_ptr()
        s.ksr_minval, s.ksr_maxval = self.minval, self.maxval
        s.ksr_channels = self.channels
        return s, buf


class NeuralMLPFunctional(XCFunctional):
    """The reference's dense XC networks with their wrappers, FP32 on the GPU.

    ``local=True``: LocalMLP (``qedft/models/networks.py:83-109``,
    ``build_local_mlp`` at ``qedft/models/classical/classical_models.py:123-174``),
    g_i = MLP(n_i / norm) at every grid point.  ``local=False``: GlobalMLP
    (``networks.py:112-138``, ``build_global_mlp`` at ``classical_models.py:177-224``),
    one g = MLP(n / norm) from the whole density (input size = the grid size).
    Wrappers (``qedft/models/wrappers.py:162-217``): ``self_interaction``
    (jax_dft's layer, u_i = beta (-v_H[n]_i / 2) + (1 - beta) g_i) and
    ``negativity`` (f = -swish(u)); a global network's output is the mean of
    f over the grid.  The network is [Dense(n_neurons), activation] x
    n_layers, Dense(1).

    ``params`` is the stax parameter tree the wrapped network's ``init_fn``
    returns (see ``qex_gb300.networks.LocalMLP`` / ``GlobalMLP``).
    """

    def __init__(self, local=True, n_neurons=64, n_layers=3, activation="tanh",
                 normalization=2.0, self_interaction=False, negativity=True, num_inputs=1):
        if activation not in N.QEX_NN_ACTIVATIONS:
            raise ValueError(f"activation {activation!r} is not on the GPU path "
                             f"(one of {sorted(N.QEX_NN_ACTIVATIONS)})")
        if not 1 <= int(n_neurons) <= N.QEX_NN_MAX_WIDTH or int(n_layers) < 1:
            raise ValueError(f"the GPU networks take 1..{N.QEX_NN_MAX_WIDTH} neurons and "
                             "at least one hidden layer")
        self.local = bool(local)
        self.kind = N.QEX_XC_LOCAL_MLP if self.local else N.QEX_XC_GLOBAL_MLP
        self.n_neurons, self.n_layers = int(n_neurons), int(n_layers)
        self.activation = activation
        self.normalization = float(normalization)
        self.self_interaction, self.negativity = bool(self_interaction), bool(negativity)
        self.num_inputs = 1 if self.local else int(num_inputs)
        self.width_padded = (self.n_neurons + 7) // 8 * 8
        self._dev = None

    def dense_layers(self, params):
        """[(W, b), ...] of the Dense layers and the self-interaction width
        (1.0 without the layer) from the wrapped network's parameter tree."""
        tree = params
        if self.negativity:
            tree = tree[0]  # stax.serial(network, negativity_transform())
        width = 1.0
        if self.self_interaction:
            # stax.serial(FanOut(2), parallel(Identity, network), self_interaction_layer)
            width = float(np.asarray(tree[2][0]))
            tree = tree[1][1]
        dense = [layer for layer in tree if len(layer) == 2]
        if len(dense) != self.n_layers + 1:
            raise ValueError(f"expected {self.n_layers + 1} Dense layers, got {len(dense)}")
        return [(np.asarray(w), np.asarray(b)) for w, b in dense], width

    def pack(self, params) -> np.ndarray:
        layers, width = self.dense_layers(params)
        H, Hp, nin = self.n_neurons, self.width_padded, self.num_inputs
        parts = []
        for li, (w, b) in enumerate(layers[:-1]):
            fin = nin if li == 0 else H
            w = np.asarray(w, np.float32).reshape(fin, H)
            wp = np.zeros((fin if li == 0 else Hp, Hp), np.float32)
            wp[:fin, :H] = w
            bp = np.zeros(Hp, np.float32)
            bp[:H] = np.asarray(b, np.float32).reshape(H)
            parts += [wp.reshape(-1), bp]
        wo, bo = layers[-1]
        wop = np.zeros(Hp, np.float32)
        wop[:H] = np.asarray(wo, np.float32).reshape(H)
        tail = np.array([float(np.asarray(bo).reshape(-1)[0]), width, 0.0, 0.0], np.float32)
        flat = np.concatenate(parts + [wop, tail])
        assert flat.size == nin * Hp + Hp + (self.n_layers - 1) * (Hp * Hp + Hp) + Hp + 4
        return np.ascontiguousarray(flat)

    def device_params(self, params):
        torch = N.require_cuda()
        flat = self.pack(params)
        key = flat.tobytes()
        if self._dev is None or self._dev[0] != key or self._dev[1].device != torch.device(
                "cuda", torch.cuda.current_device()):
            self._dev = (key, torch.as_tensor(flat, device="cuda"))
        return self._dev[1]

    def spec(self, params, convention):
        if params is None:
            raise ValueError("NeuralMLPFunctional needs params")
        if not self.local and convention != N.QEX_XC_AMPLITUDE:
            raise ValueError("a global network is an amplitude-encoded functional "
                             "(kohn_sham_amplitude_encoded)")
        s, _ = super().spec(params, convention)
        buf = self.device_params(params)
        s.nn_params = buf.data_ptr()
        s.nn_width = self.width_padded
        s.nn_layers = self.n_layers
        s.nn_activation = N.QEX_NN_ACTIVATIONS[self.activation]
        s.nn_inputs = self.num_inputs
        s.nn_flags = ((N.QEX_NN_SELF_INTERACTION if self.self_interaction else 0)
                      | (N.QEX_NN_NEGATIVITY if self.negativity else 0))
        s.normalization = self.normalization
        return s, buf


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
