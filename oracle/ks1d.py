"""NumPy float64 restatement of the 1D Kohn-Sham SCF path (test oracle).

Test infrastructure only: the CUDA product path never imports this module.

Every function restates the arithmetic of the reference (qedft, which calls the
jax_dft primitives at git rev c27ed001a50cf23f8db4d8ab4c537a36a72982de).  The
reference file:line each one follows is given in its docstring.  jax_dft is
not vendored in the reference tree; its functions are restated from their
call sites and tests in qedft and from the published algorithm.

Conventions shared with the CUDA path:
  * ``stencil`` is the kinetic finite-difference half-bandwidth in points:
    5 -> fourth-order five-point Laplacian (jax_dft ``discrete_laplacian``, what
    the reference uses), 3 -> second-order three-point Laplacian.
  * ``convention='amplitude'`` is qedft's amplitude-encoded XC
    (E_xc = dx*sum(f(n)), v_xc = dE_xc/dn, which carries a factor dx;
    ``qedft/train/od/scf.py:32-76``); ``convention='local'`` is jax_dft's
    local XC (E_xc = dx*sum(eps(n)*n), v_xc = (dE_xc/dn)/dx).
"""

from __future__ import annotations

import dataclasses
import math
from typing import Callable

import numpy as np

# Exponential-Coulomb interaction constants.  Pinned by
# data/od/*/external_potentials.npy (chain potential reproduced to ~2e-15).
EXPONENTIAL_COULOMB_AMPLITUDE = 1.071295
EXPONENTIAL_COULOMB_KAPPA = 1.0 / 2.385345


# ----------------------------------------------------------------------------
# Grid, interactions, external potential
# ----------------------------------------------------------------------------

def get_dx(grids: np.ndarray) -> float:
    """Grid spacing (jax_dft ``utils.get_dx``; used at ``qedft/train/od/scf.py:50,194``)."""
    grids = np.asarray(grids)
    if grids.ndim != 1:
        raise ValueError("grids must be one-dimensional")
    return float((np.amax(grids) - np.amin(grids)) / (grids.size - 1))


def exponential_coulomb(displacements, amplitude=EXPONENTIAL_COULOMB_AMPLITUDE,
                        kappa=EXPONENTIAL_COULOMB_KAPPA):
    """A*exp(-kappa*|d|) (jax_dft ``utils.exponential_coulomb``; ``qedft/train/od/train.py:108``)."""
    return amplitude * np.exp(-np.abs(displacements) * kappa)


def soft_coulomb(displacements, soften_factor=1.0):
    """1/sqrt(d^2+s) (jax_dft ``utils.soft_coulomb``; ``tests/test_scf_od.py:118``)."""
    return 1.0 / np.sqrt(np.square(displacements) + soften_factor)


def gaussian(grids, center, sigma=1.0):
    """Normalised Gaussian (jax_dft ``utils.gaussian``; ``tests/test_scf_od.py:155``)."""
    grids = np.asarray(grids, dtype=np.float64)
    return (1.0 / math.sqrt(2.0 * math.pi) * np.exp(-0.5 * ((grids - center) / sigma) ** 2)
            / sigma)


def get_atomic_chain_potential(grids, locations, nuclear_charges, interaction_fn):
    """v_ext(x) = -sum_j Z_j K(x - R_j).

    jax_dft ``utils.get_atomic_chain_potential`` as called at
    ``qedft/train/od/jit_scf.py:219-224`` and ``qedft/train/od/scf.py:490-495``.
    """
    grids = np.asarray(grids, dtype=np.float64)
    locations = np.asarray(locations, dtype=np.float64).reshape(-1)
    charges = np.asarray(nuclear_charges, dtype=np.float64).reshape(-1)
    disp = grids[None, :] - locations[:, None]
    return -(charges[:, None] * interaction_fn(disp)).sum(axis=0)


# ----------------------------------------------------------------------------
# Kinetic operator and the non-interacting solve
# ----------------------------------------------------------------------------

def discrete_laplacian(num_grids: int, stencil: int = 5) -> np.ndarray:
    """Dense finite-difference Laplacian (unit spacing).

    stencil=5 is jax_dft ``scf.discrete_laplacian`` (fourth order:
    -1/12, 4/3, -5/2, 4/3, -1/12), used by ``qedft/train/od/scf.py:185-195``.
    stencil=3 is the second-order (1, -2, 1) operator.
    """
    if stencil == 5:
        coeffs = (-2.5, 4.0 / 3.0, -1.0 / 12.0)
    elif stencil == 3:
        coeffs = (-2.0, 1.0)
    else:
        raise ValueError(f"stencil must be 3 or 5, got {stencil}")
    mat = np.diag(np.full(num_grids, coeffs[0]))
    for off, c in enumerate(coeffs[1:], start=1):
        mat += np.diag(np.full(num_grids - off, c), k=off)
        mat += np.diag(np.full(num_grids - off, c), k=-off)
    return mat


def get_kinetic_matrix(grids, stencil: int = 5) -> np.ndarray:
    """T = -1/2 L / dx^2 (``qedft/train/od/scf.py:185-195``)."""
    dx = get_dx(grids)
    return -0.5 * discrete_laplacian(np.asarray(grids).size, stencil) / (dx * dx)


def wavefunctions_to_density(num_electrons: int, wavefunctions: np.ndarray, grids) -> np.ndarray:
    """Normalise, repeat each orbital for two spins, sum the first Ne.

    ``qedft/train/od/scf.py:198-213``.  ``wavefunctions`` is (num_states, N).
    """
    wf = np.asarray(wavefunctions, dtype=np.float64)[:num_electrons]
    wf = wf / np.sqrt(np.sum(wf ** 2, axis=1, keepdims=True) * get_dx(grids))
    intensities = np.repeat(wf ** 2, repeats=2, axis=0)
    return np.sum(intensities[:num_electrons], axis=0)


def get_total_eigen_energies(num_electrons: int, eigen_energies: np.ndarray) -> float:
    """Sum of the first Ne spin-repeated eigenvalues (jax_dft; ``qedft/train/od/scf.py:245-248``)."""
    return float(np.sum(np.repeat(eigen_energies, repeats=2)[:num_electrons]))


def get_gap(num_electrons: int, eigen_energies: np.ndarray) -> float:
    """LUMO - HOMO on the spin-repeated spectrum (jax_dft; ``qedft/train/od/scf.py:249``).

    For odd Ne the HOMO orbital is half filled, so LUMO == HOMO and the gap is 0.
    """
    rep = np.repeat(eigen_energies, repeats=2)
    return float(rep[num_electrons] - rep[num_electrons - 1])


def _lowest_eigenpairs(potential, grids, count: int, stencil: int, method: str):
    """Lowest ``count`` eigenpairs of T + diag(v).

    method='dense' is the reference algorithm (``jnp.linalg.eigh`` of the dense
    Hamiltonian, ``qedft/train/od/scf.py:235-239``); method='banded' uses LAPACK
    banded selected-eigenpair routines (same mathematics, faster for tests).
    Returns (eigenvalues (count,), eigenvectors (count, N)).
    """
    potential = np.asarray(potential, dtype=np.float64)
    n = potential.size
    if method == "dense":
        ham = get_kinetic_matrix(grids, stencil) + np.diag(potential)
        w, v = np.linalg.eigh(ham)
        return w[:count], v[:, :count].T
    if method == "banded":
        import scipy.linalg as sla
        dx = get_dx(grids)
        if stencil == 5:
            lap = (-2.5, 4.0 / 3.0, -1.0 / 12.0)
        else:
            lap = (-2.0, 1.0)
        b = len(lap) - 1
        band = np.zeros((b + 1, n))
        band[0] = -0.5 * lap[0] / (dx * dx) + potential
        for off in range(1, b + 1):
            band[off, : n - off] = -0.5 * lap[off] / (dx * dx)
        w, v = sla.eig_banded(band, lower=True, select="i", select_range=(0, count - 1))
        return w, v.T
    raise ValueError(method)


def solve_noninteracting_system(external_potential, num_electrons: int, grids,
                                stencil: int = 5, method: str = "dense"):
    """Density, total eigen-energy and gap of T + diag(v).

    ``qedft/train/od/scf.py:233-250`` (jax_dft ``solve_noninteracting_system``).
    """
    count = num_electrons // 2 + 1  # eigenvalues needed for the sum and the gap
    count = max(count, (num_electrons + 1) // 2)
    w, vecs = _lowest_eigenpairs(external_potential, grids, count, stencil, method)
    density = wavefunctions_to_density(num_electrons, vecs, grids)
    return density, get_total_eigen_energies(num_electrons, w), get_gap(num_electrons, w)


# ----------------------------------------------------------------------------
# Hartree and external energies
# ----------------------------------------------------------------------------

def get_hartree_potential(density, grids, interaction_fn):
    """v_H(x_i) = dx * sum_j n_j K(x_i - x_j), N x N kernel materialised.

    ``qedft/train/od/scf.py:303-308``.
    """
    grids = np.asarray(grids, dtype=np.float64)
    kern = interaction_fn(grids[None, :] - grids[:, None])
    return kern @ np.asarray(density, dtype=np.float64) * get_dx(grids)


def get_hartree_energy(density, grids, interaction_fn):
    """E_H = 1/2 dx^2 sum_ij n_i n_j K_ij (``qedft/train/od/scf.py:271-283``)."""
    grids = np.asarray(grids, dtype=np.float64)
    n = np.asarray(density, dtype=np.float64)
    kern = interaction_fn(grids[None, :] - grids[:, None])
    return float(0.5 * n @ kern @ n * get_dx(grids) ** 2)


def get_external_potential_energy(external_potential, density, grids):
    """dx * <n, v> (jax_dft; ``qedft/train/od/scf.py:139-143``)."""
    return float(np.dot(density, external_potential) * get_dx(grids))


# ----------------------------------------------------------------------------
# Exchange-correlation functionals
# ----------------------------------------------------------------------------

class PointwiseXC:
    """Base for XC functionals: per-point values f(n) and vector-Jacobian products."""

    def values(self, density: np.ndarray) -> np.ndarray:
        raise NotImplementedError

    def vjp(self, density: np.ndarray, cotangent: np.ndarray) -> np.ndarray:
        """Return J^T g with J = d values / d density."""
        raise NotImplementedError


class PowerXC(PointwiseXC):
    """f(n) = a * (n + shift)^p; with a=-0.73855, p=1/3 this is the 3D-LDA
    exchange test functional of ``tests/test_scf_od.py:46-48,127-129``."""

    def __init__(self, coefficient=-0.73855, power=1.0 / 3.0, shift=0.0):
        self.a, self.p, self.shift = float(coefficient), float(power), float(shift)

    def values(self, density):
        return self.a * (np.asarray(density) + self.shift) ** self.p

    def vjp(self, density, cotangent):
        return cotangent * self.a * self.p * (np.asarray(density) + self.shift) ** (self.p - 1.0)


class LDAExpCoulomb(PointwiseXC):
    """Exponential-Coulomb uniform-gas LDA: eps_xc(n) = eps_x(n) + eps_c(n).

    jax_dft ``xc.get_lda_xc_energy_density_fn`` (called at
    ``qedft/train/od/eval.py:79``), restated from the published fit of Baker
    et al., PRB 91, 235141 (2015).  Parity unpinned (no reference test holds a
    value).  y = pi*n/kappa;
      eps_x = A/(2 pi) * (ln(1+y^2)/y - 2 atan y)          (y > 1e-15)
            = A/(2 pi) * (-y + y^3/6)                      (otherwise)
      eps_c = -A y / pi / P(y),
      P(y)  = 2 - 1.00077 y^.5 + 6.26099 y - 11.9041 y^1.5
              + 9.62614 y^2 - 1.48334 y^2.5 + pi kappa^2/A y^3.
    """

    ALPHA, BETA, GAMMA, DELTA, ETA, SIGMA, NU = (2.0, -1.00077, 6.26099, -11.9041,
                                                 9.62614, -1.48334, 1.0)

    def __init__(self, amplitude=EXPONENTIAL_COULOMB_AMPLITUDE, kappa=EXPONENTIAL_COULOMB_KAPPA):
        self.A, self.kappa = float(amplitude), float(kappa)

    def _poly(self, y):
        s = np.sqrt(y)
        c3 = self.NU * math.pi * self.kappa ** 2 / self.A
        p = (self.ALPHA + self.BETA * s + self.GAMMA * y + self.DELTA * y * s + self.ETA * y * y
             + self.SIGMA * y * y * s + c3 * y ** 3)
        dp = (0.5 * self.BETA / np.where(s > 0, s, 1.0) + self.GAMMA + 1.5 * self.DELTA * s
              + 2.0 * self.ETA * y + 2.5 * self.SIGMA * y * s + 3.0 * c3 * y * y)
        return p, dp

    def _eps_and_deps_dy(self, density):
        n = np.asarray(density, dtype=np.float64)
        y = math.pi * n / self.kappa
        big = y > 1e-15
        ys = np.where(big, y, 1.0)
        ax = self.A / (2.0 * math.pi)
        ex = np.where(big, ax * (np.log1p(ys * ys) / ys - 2.0 * np.arctan(ys)),
                      ax * (-y + y ** 3 / 6.0))
        dex = np.where(big, -ax * np.log1p(ys * ys) / (ys * ys), ax * (-1.0 + 0.5 * y * y))
        pos = y > 0
        yc = np.where(pos, y, 1.0)
        p, dp = self._poly(yc)
        ec = np.where(pos, -self.A * yc / math.pi / p, 0.0)
        dec = np.where(pos, -self.A / math.pi * (p - yc * dp) / (p * p),
                       -self.A / math.pi / self.ALPHA)
        return ex + ec, (dex + dec), y

    def values(self, density):
        return self._eps_and_deps_dy(density)[0]

    def vjp(self, density, cotangent):
        _, deps_dy, _ = self._eps_and_deps_dy(density)
        return cotangent * deps_dy * (math.pi / self.kappa)


def _silu(x):
    return x / (1.0 + np.exp(-x))


def _silu_grad(x):
    s = 1.0 / (1.0 + np.exp(-x))
    return s * (1.0 + x * (1.0 - s))


class WindowMLP(PointwiseXC):
    """Per-point MLP on a window of the density: eps_i = MLP(n[i-h..i+h] / norm).

    Local neural XC of the batched 1D configuration (window 17, two SiLU hidden
    layers of 16, one output), following the local-MLP form of
    ``qedft/models/classical/classical_models.py:123-174`` (input divided by
    ``density_normalization_factor``, the same dense stack applied at every grid
    point) with a zero-padded window in place of the single point.
    ``layers`` is a list of (W (in, out), b (out,)) pairs applied as x@W+b with
    SiLU between layers (stax ``Dense`` convention).  ``dtype`` selects float32
    (the arithmetic the GPU uses) or float64.
    """

    def __init__(self, layers, window=17, normalization=2.0, dtype=np.float64):
        self.layers = [(np.asarray(w, dtype=dtype), np.asarray(b, dtype=dtype)) for w, b in layers]
        self.window = int(window)
        if self.window % 2 != 1:
            raise ValueError("window must be odd")
        self.half = self.window // 2
        self.norm = float(normalization)
        self.dtype = dtype

    def _windows(self, density):
        n = np.asarray(density, dtype=self.dtype) / self.dtype(self.norm)
        pad = np.concatenate([np.zeros(self.half, self.dtype), n, np.zeros(self.half, self.dtype)])
        idx = np.arange(n.size)[:, None] + np.arange(self.window)[None, :]
        return pad[idx]

    def _forward(self, density):
        x = self._windows(density)
        pre = []
        for li, (w, b) in enumerate(self.layers):
            z = x @ w + b
            if li < len(self.layers) - 1:
                pre.append(z)
                x = _silu(z)
            else:
                x = z
        return x[:, 0], pre

    def values(self, density):
        return self._forward(density)[0].astype(np.float64)

    def input_gradients(self, density):
        """(N, window) array of d eps_i / d window_i (already divided by norm)."""
        _, pre = self._forward(density)
        g = np.broadcast_to(self.layers[-1][0][:, 0], (pre[-1].shape[0], self.layers[-1][0].shape[0]))
        for li in range(len(self.layers) - 2, -1, -1):
            g = g * _silu_grad(pre[li])
            g = g @ self.layers[li][0].T
        return g / self.dtype(self.norm)

    def vjp(self, density, cotangent):
        grad = self.input_gradients(density).astype(np.float64)
        cot = np.asarray(cotangent, dtype=np.float64)
        n = grad.shape[0]
        out = np.zeros(n + 2 * self.half)
        contrib = grad * cot[:, None]
        for k in range(self.window):
            out[k: k + n] += contrib[:, k]
        return out[self.half: self.half + n]


class KSRGlobalConv(PointwiseXC):
    """The Kohn-Sham-regularizer global-local convolutional XC network (FP64).

    ``qedft/models/classical/global_ksr_model.py:32-80``
    (``create_ksr_model_from_config``) builds, from jax_dft ``neural_xc``:

      1. ``global_conv_block(num_global_filters)``: FanOut(2) ->
         parallel(Identity, exponential_global_convolution(num_global_filters - 1))
         -> FanInConcat; channel 0 is the density itself and channel c >= 1 is
         G_c(x_i) = dx * sum_j n_j exp(-|x_i - x_j| / w_c) / (2 w_c) over the grid
         points, with w_c = minval + (maxval - minval) * sigmoid(eta_c);
      2. ``num_local_conv_layers`` times: bias-free 1D convolution of width 3,
         SAME (zero) padding, cross-correlation with kernel W (3, C_in, C_out),
         then swish (x * sigmoid(x));
      3. a bias-free width-1 convolution to one channel, then the negativity
         transform -swish(y);
      4. ``wrap_network_with_self_interaction_layer`` with exponential_coulomb:
         eps = beta * (-v_H[n] / 2) + (1 - beta) * network(n), where
         beta = exp(-((dx sum n - 1) / width)^2) and width is a parameter;
      5. ``global_functional``: eps over the grid from the density vector.

    jax_dft ``neural_xc`` is not in the reference tree; the architecture above
    is restated from the published model (Li et al., PRL 126, 036401) and
    pinned by the trained parameters shipped at ``data/od/h2/h2_optimal.pkl``
    (their nesting is exactly global block, conv, act, conv, act, conv,
    transform; the self-interaction width is the last leaf): with them the
    jax_dft local-convention SCF of ``qedft/train/od/train.py:84-125``
    (reflection symmetry on, 15 iterations, one mixing step) reproduces the
    reference's exact H2 energies ``data/od/h2/total_energies.npy`` to about
    1 mHa at bond lengths 0.6-2.7 bohr, which no other reading of the layer
    list does (a missing or softplus transform misses by 0.1-0.6 Ha).

    ``params`` is a dict with keys ``eta`` (C-1,), ``conv`` (list of (3, C, C)
    kernels), ``out`` (1, C, 1), ``width`` (scalar), ``minval``, ``maxval``.
    """

    def __init__(self, grids, params, dtype=np.float64):
        self.grids = np.asarray(grids, dtype=np.float64)
        self.dx = get_dx(self.grids)
        self.dtype = dtype
        self.eta = np.asarray(params["eta"], np.float64)
        self.conv = [np.asarray(w, dtype) for w in params["conv"]]
        self.out = np.asarray(params["out"], dtype)
        self.width = float(params["width"])
        lo, hi = float(params.get("minval", 0.1)), float(params.get("maxval", 2.385345))
        self.widths = lo + (hi - lo) / (1.0 + np.exp(-self.eta))
        d = np.abs(self.grids[None, :] - self.grids[:, None])
        # (N, N, C-1) global kernels, dx included
        self.kern = (np.exp(-d[..., None] / self.widths) / (2.0 * self.widths) * self.dx).astype(dtype)

    @staticmethod
    def _sig(x):
        return 1.0 / (1.0 + np.exp(-x))

    @classmethod
    def _swish(cls, x):
        return x * cls._sig(x)

    @classmethod
    def _dswish(cls, x):
        s = cls._sig(x)
        return s * (1.0 + x * (1.0 - s))

    @staticmethod
    def _conv(a, w):
        """SAME cross-correlation: out[i] = sum_t a[i + t - h] @ w[t]."""
        k, h, n = w.shape[0], w.shape[0] // 2, a.shape[0]
        pad = np.concatenate([np.zeros((h, a.shape[1]), a.dtype), a, np.zeros((h, a.shape[1]), a.dtype)])
        out = np.zeros((n, w.shape[2]), a.dtype)
        for t in range(k):
            out += pad[t:t + n] @ w[t]
        return out

    @staticmethod
    def _conv_t(d, w):
        """Adjoint of ``_conv`` with respect to its input."""
        k, h, n = w.shape[0], w.shape[0] // 2, d.shape[0]
        out = np.zeros((n + 2 * h, w.shape[1]), d.dtype)
        for t in range(k):
            out[t:t + n] += d @ w[t].T
        return out[h:h + n]

    def _forward(self, density):
        n64 = np.asarray(density, np.float64)
        n = n64.astype(self.dtype)
        f = np.concatenate([n[:, None], np.einsum("j,jic->ic", n, self.kern)], axis=1)
        zs, a = [], f
        for w in self.conv:
            z = self._conv(a, w)
            zs.append(z)
            a = self._swish(z)
        y = self._conv(a, self.out)[:, 0]
        o = -self._swish(y)
        integral = float(np.sum(n64) * self.dx)
        beta = math.exp(-((integral - 1.0) / self.width) ** 2)
        h = -0.5 * get_hartree_potential(n64, self.grids, exponential_coulomb)
        eps = beta * h + (1.0 - beta) * o.astype(np.float64)
        return eps, (zs, y, o, beta, h, integral)

    def values(self, density):
        return self._forward(density)[0]

    def vjp(self, density, cotangent):
        _, (zs, y, o, beta, h, integral) = self._forward(density)
        g = np.asarray(cotangent, np.float64)
        dbeta = beta * (-2.0 * (integral - 1.0) / self.width ** 2)
        dn = np.full(g.size, float(np.dot(g, h - o)) * dbeta * self.dx)
        dn += -0.5 * beta * get_hartree_potential(g, self.grids, exponential_coulomb)
        dy = ((1.0 - beta) * g).astype(self.dtype) * -self._dswish(y)
        da = dy[:, None] * self.out[0, :, 0][None, :]
        for li in range(len(self.conv) - 1, -1, -1):
            dz = da * self._dswish(zs[li])
            da = self._conv_t(dz, self.conv[li])
        dn += da[:, 0] + np.einsum("ic,jic->j", da[:, 1:], self.kern)
        return dn


_NN_ACTIVATIONS = {
    # name: (f(z), f'(z)), the stax layers of qedft/models/classical/classical_models.py:37-47
    "tanh": (np.tanh, lambda z: 1.0 - np.tanh(z) ** 2),
    "relu": (lambda z: np.maximum(z, 0.0), lambda z: (z > 0).astype(z.dtype)),
    "softplus": (lambda z: np.logaddexp(z, 0.0), lambda z: 0.5 * (1.0 + np.tanh(0.5 * z))),
    "sigmoid": (lambda z: 0.5 * (1.0 + np.tanh(0.5 * z)),
                lambda z: 0.25 * (1.0 - np.tanh(0.5 * z) ** 2)),
    "elu": (lambda z: np.where(z > 0, z, np.expm1(np.minimum(z, 0.0))),
            lambda z: np.where(z > 0, 1.0, np.exp(np.minimum(z, 0.0)))),
    "leaky_relu": (lambda z: np.where(z >= 0, z, 0.01 * z), lambda z: np.where(z >= 0, 1.0, 0.01)),
    "selu": (lambda z: 1.0507009873554805 * np.where(
        z > 0, z, 1.6732632423543772 * np.expm1(np.minimum(z, 0.0))),
             lambda z: 1.0507009873554805 * np.where(
        z > 0, 1.0, 1.6732632423543772 * np.exp(np.minimum(z, 0.0)))),
    "gelu": (lambda z: 0.5 * z * (1.0 + np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3))),
             lambda z: (0.5 * (1.0 + np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))
                        + 0.5 * z * (1.0 - np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)) ** 2)
                        * 0.7978845608028654 * (1.0 + 3 * 0.044715 * z * z))),
}


class DenseNetworkXC(PointwiseXC):
    """The reference's dense XC networks with their wrappers.

    Network: x -> [Dense(H), activation] x L -> Dense(1), x = n / norm
    (``build_mlp_layers``, ``qedft/models/classical/classical_models.py:77-115``):
      * local (``build_local_mlp``, :123-174; ``LocalMLP``,
        ``qedft/models/networks.py:83-109``): g_i = MLP(n_i / norm) per point;
      * global (``build_global_mlp``, :177-224; ``GlobalMLP``, networks.py:112-138):
        g = MLP(n / norm) on the whole density.
    Wrappers (``qedft/models/wrappers.py:162-217``), in the reference's order:
      * self-interaction (jax_dft ``wrap_network_with_self_interaction_layer``
        with exponential_coulomb): u_i = beta (-v_H[n]_i / 2) + (1 - beta) g_i,
        beta = exp(-((dx sum n - 1) / width)^2);
      * negativity (jax_dft ``negativity_transform``): f = -swish(u);
      * global networks: the mean of f over the grid (``global_apply_fn``),
        returned here as per-point values f_i / N (their sum is the scalar).
    ``layers``: [(W (in, out), b (out,)), ...] of the Dense layers; ``dtype``
    is the network's arithmetic (float32 as on the GPU, or float64); the
    wrappers run in float64.
    """

    def __init__(self, grids, layers, activation="tanh", normalization=2.0, local=True,
                 self_interaction=False, negativity=True, width=1.0, dtype=np.float64):
        self.grids = np.asarray(grids, dtype=np.float64)
        self.dx = get_dx(self.grids)
        self.layers = [(np.asarray(w, dtype), np.asarray(b, dtype).reshape(-1)) for w, b in layers]
        self.act, self.dact = _NN_ACTIVATIONS[activation]
        self.norm = float(normalization)
        self.local, self.si, self.neg = bool(local), bool(self_interaction), bool(negativity)
        self.width = float(width)
        self.dtype = dtype

    def _network(self, n64):
        """g (per point, or a scalar) and its input gradient (per point)."""
        x = (n64.astype(self.dtype) / self.dtype(self.norm))
        x = x[:, None] if self.local else x[None, :]
        zs, a = [], x
        for w, b in self.layers[:-1]:
            z = a @ w + b
            zs.append(z)
            a = self.act(z)
        w, b = self.layers[-1]
        g = (a @ w + b)[:, 0]
        # reverse pass of the scalar outputs (one row per point, or one row)
        d = np.broadcast_to(w[:, 0], a.shape).astype(self.dtype)
        for li in range(len(zs) - 1, -1, -1):
            d = d * self.dact(zs[li])
            d = d @ self.layers[li][0].T
        gx = d / self.dtype(self.norm)
        if self.local:
            return g.astype(np.float64), gx[:, 0].astype(np.float64)
        return float(g[0]), gx[0].astype(np.float64)

    def _forward(self, density):
        n = np.asarray(density, np.float64)
        g, gx = self._network(n)
        q = float(np.sum(n) * self.dx)
        beta = math.exp(-((q - 1.0) / self.width) ** 2) if self.si else 0.0
        vh = get_hartree_potential(n, self.grids, exponential_coulomb) if self.si else 0.0
        u = -0.5 * beta * vh + (1.0 - beta) * g if self.si else g * np.ones_like(n)
        if self.neg:
            s = 1.0 / (1.0 + np.exp(-u))
            f, fp = -u * s, -(s + u * s * (1.0 - s))
        else:
            f, fp = u, np.ones_like(u)
        scale = 1.0 if self.local else 1.0 / n.size
        return f * scale, (g, gx, q, beta, vh, fp * scale)

    def values(self, density):
        return self._forward(density)[0]

    def vjp(self, density, cotangent):
        _, (g, gx, q, beta, vh, fps) = self._forward(density)
        c = np.asarray(cotangent, np.float64) * fps
        keep = (1.0 - beta) if self.si else 1.0
        out = keep * (c * gx if self.local else np.sum(c) * gx)
        if self.si:
            dbeta = beta * (-2.0 * (q - 1.0) / self.width ** 2) * self.dx
            out = out - 0.5 * beta * get_hartree_potential(c, self.grids, exponential_coulomb)
            out = out + float(np.dot(c, -0.5 * vh - g)) * dbeta
        return out


def ksr_params_from_tree(tree, minval=0.1, maxval=2.385345):
    """The dict form of ``KSRGlobalConv`` params from the stax parameter tree of
    ``create_ksr_model_from_config`` (the nesting of ``data/od/h2/h2_optimal.pkl``:
    [(), ((), [global block, (W1,), (), (W2,), (), (W3,), ()]), (width,)])."""
    net = tree[1][1]
    eta = np.asarray(net[0][1][1][0][0], np.float64)
    convs = [np.asarray(layer[0], np.float64) for layer in net[1:-2] if len(layer) == 1]
    out = np.asarray(net[-2][0], np.float64)
    width = float(np.asarray(tree[2][0]))
    return {"eta": eta, "conv": convs, "out": out, "width": width, "minval": minval,
            "maxval": maxval}


def _flip_avg(x):
    """(x + reverse(x)) / 2 about the grid centre (jax_dft ``jit_scf._flip_and_average_on_center``,
    used at ``qedft/train/od/jit_scf.py:76-77``)."""
    return 0.5 * (x + x[::-1])


def xc_energy(density, xc: PointwiseXC, grids, convention: str, reflection: bool = False):
    """E_xc for either convention (amplitude: ``qedft/train/od/scf.py:32-50``)."""
    dx = get_dx(grids)
    n = np.asarray(density, dtype=np.float64)
    if convention == "amplitude":
        return float(np.sum(xc.values(n)) * dx)
    if reflection:
        eps = _flip_avg(xc.values(_flip_avg(n)))
    else:
        eps = xc.values(n)
    return float(np.dot(eps, n) * dx)


def xc_potential(density, xc: PointwiseXC, grids, convention: str, reflection: bool = False):
    """v_xc = dE_xc/dn (amplitude, ``qedft/train/od/scf.py:53-76``) or (dE_xc/dn)/dx (local)."""
    dx = get_dx(grids)
    n = np.asarray(density, dtype=np.float64)
    if convention == "amplitude":
        return dx * xc.vjp(n, np.ones_like(n))
    if reflection:
        s = _flip_avg(n)
        return _flip_avg(xc.values(s)) + _flip_avg(xc.vjp(s, s))
    return xc.values(n) + xc.vjp(n, n)


def xc_energy_density(density, xc: PointwiseXC, convention: str, reflection: bool = False):
    """The state's ``xc_energy_density`` field: the per-point eps (local) or the
    summed network output (amplitude, ``qedft/train/od/jit_scf.py:37``)."""
    n = np.asarray(density, dtype=np.float64)
    if convention == "amplitude":
        return float(np.sum(xc.values(n)))
    if reflection:
        return _flip_avg(xc.values(_flip_avg(n)))
    return xc.values(n)


# ----------------------------------------------------------------------------
# One Kohn-Sham iteration and the SCF drivers
# ----------------------------------------------------------------------------

@dataclasses.dataclass
class IterationResult:
    density: np.ndarray
    total_energy: float
    hartree_potential: np.ndarray
    xc_potential: np.ndarray
    xc_energy_density: object
    gap: float


def kohn_sham_iteration(density, external_potential, grids, num_electrons, xc, interaction_fn,
                        enforce_reflection_symmetry=False, convention="amplitude", stencil=5,
                        method="dense") -> IterationResult:
    """One KS iteration.

    Amplitude convention: ``qedft/train/od/jit_scf.py:14-86`` (same arithmetic as
    ``qedft/train/od/scf.py:79-177``).  Local convention: jax_dft
    ``jit_scf._kohn_sham_iteration`` (selected at ``qedft/train/od/train.py:117-121``),
    whose reflection option also symmetrises the XC functional.
    """
    grids = np.asarray(grids, dtype=np.float64)
    reflect_xc = enforce_reflection_symmetry and convention == "local"
    v_h = get_hartree_potential(density, grids, interaction_fn)
    v_xc = xc_potential(density, xc, grids, convention, reflect_xc)
    v_ks = v_h + v_xc + external_potential
    eps = xc_energy_density(density, xc, convention, reflect_xc)
    n_out, tee, gap = solve_noninteracting_system(v_ks, num_electrons, grids, stencil, method)
    total = (tee - get_external_potential_energy(v_ks, n_out, grids)
             + get_hartree_energy(n_out, grids, interaction_fn)
             + xc_energy(n_out, xc, grids, convention, reflect_xc)
             + get_external_potential_energy(external_potential, n_out, grids))
    if enforce_reflection_symmetry:
        n_out = _flip_avg(n_out)
    return IterationResult(n_out, total, v_h, v_xc, eps, gap)


def connection_weights(num_iterations: int, num_mixing_iterations: int) -> np.ndarray:
    """Row t averages the last min(t+1, m) density differences.

    jax_dft ``jit_scf._connection_weights`` as used at ``qedft/train/od/jit_scf.py:162,180``
    (the Python twin ``qedft/train/od/scf.py:547-555`` averages ``differences[-m:]``).
    """
    mask = np.triu(np.tril(np.ones((num_iterations, num_iterations))),
                   k=-num_mixing_iterations + 1)
    return mask / mask.sum(axis=1, keepdims=True)


def kohn_sham(locations, nuclear_charges, num_electrons, num_iterations, grids, xc,
              interaction_fn=exponential_coulomb, initial_density=None, alpha=0.5,
              alpha_decay=0.9, enforce_reflection_symmetry=False, num_mixing_iterations=2,
              density_mse_converge_tolerance=-1.0, convention="amplitude", stencil=5,
              driver="jit", method="dense"):
    """Full SCF; returns a dict of stacked per-iteration fields.

    driver='jit' follows ``qedft/train/od/jit_scf.py:143-244`` (lax.scan body:
    converged-skip, mixing with connection weights, converged = MSE(mixed - old)
    < tol, alpha decays every step).  driver='python' follows
    ``qedft/train/od/scf.py:434-560`` (converged = MSE(unmixed - old) < tol, early
    stop pads with the converged state, alpha decays on active steps only,
    default initial density = non-interacting solution of v_ext).
    """
    grids = np.asarray(grids, dtype=np.float64)
    n_grid = grids.size
    v_ext = get_atomic_chain_potential(grids, locations, nuclear_charges, interaction_fn)
    if initial_density is None:
        if driver == "jit":
            raise ValueError("the jit driver requires initial_density")
        initial_density, _, _ = solve_noninteracting_system(v_ext, num_electrons, grids,
                                                            stencil, method)
    density = np.array(initial_density, dtype=np.float64)
    weights = connection_weights(num_iterations, num_mixing_iterations)
    diffs = np.zeros((num_iterations, n_grid))
    state = dict(density=density, total_energy=np.inf, hartree_potential=np.zeros(n_grid),
                 xc_potential=np.zeros(n_grid), xc_energy_density=0.0, gap=0.0, converged=False)
    out = {k: [] for k in state}
    converged = False
    py_diffs = []
    for idx in range(num_iterations):
        old = state
        if converged:
            state = dict(old)
            state["converged"] = True
        else:
            res = kohn_sham_iteration(old["density"], v_ext, grids, num_electrons, xc,
                                      interaction_fn, enforce_reflection_symmetry, convention,
                                      stencil, method)
            diff = res.density - old["density"]
            state = dict(old)
            state.update(total_energy=res.total_energy, hartree_potential=res.hartree_potential,
                         xc_potential=res.xc_potential, xc_energy_density=res.xc_energy_density,
                         gap=res.gap)
            if driver == "jit":
                diffs[idx] = diff
                state["density"] = old["density"] + alpha * (weights[idx] @ diffs)
            else:
                py_diffs.append(diff)
                if np.mean(np.square(diff)) < density_mse_converge_tolerance:
                    converged = True
                state["converged"] = converged
                state["density"] = old["density"] + alpha * np.mean(
                    py_diffs[-num_mixing_iterations:], axis=0)
                alpha *= alpha_decay
        if driver == "jit":
            converged = bool(np.mean(np.square(state["density"] - old["density"]))
                             < density_mse_converge_tolerance)
            alpha *= alpha_decay
        for k in out:
            out[k].append(state[k])
    result = {k: np.array(v) for k, v in out.items()}
    result["external_potential"] = v_ext
    return result


# ----------------------------------------------------------------------------
# Loss of the differentiation configuration
# ----------------------------------------------------------------------------

def config3_loss(energies, densities, target_energies, target_densities, grids,
                 density_weight=0.1):
    """sum_b (E_b - E_b^t)^2 + w * sum_b ||n_b - n_b^t||^2 dx (final iterate)."""
    dx = get_dx(grids)
    e = np.asarray(energies) - np.asarray(target_energies)
    d = np.asarray(densities) - np.asarray(target_densities)
    return float(np.sum(e * e) + density_weight * np.sum(d * d) * dx)


def reference_training_loss(energies, final_densities, target_energy, target_density, grids,
                            num_electrons, discount=0.9, ks_iter_to_ignore=10):
    """The reference's training loss, ``qedft/train/od/train.py:296-318``: the
    discounted trajectory MSE of the energies from ``ks_iter_to_ignore`` on,
    over Ne, plus the MSE of the final densities times dx N, over Ne (jax_dft
    ``losses``, restated in ``qedft/train/od/losses_no_jit.py:8-102``)."""
    grids = np.asarray(grids, dtype=np.float64)
    e = np.asarray(energies, dtype=np.float64)[:, ks_iter_to_ignore:]
    loss = trajectory_mse(target_energy, e, discount) / num_electrons
    d = np.asarray(target_density, dtype=np.float64) - np.asarray(final_densities, dtype=np.float64)
    loss += float(np.mean(d * d)) * get_dx(grids) * grids.size / num_electrons
    return float(loss)


def trajectory_mse(target, predict, discount):
    """Discounted trajectory MSE (jax_dft ``losses.trajectory_mse``; ``qedft/train/od/train.py:296-302``).

    predict is (batch, steps); the step weights are discount**(steps-1-t); the
    error is averaged over the batch and summed over steps.
    """
    predict = np.asarray(predict, dtype=np.float64)
    target = np.asarray(target, dtype=np.float64)
    steps = predict.shape[1]
    w = discount ** np.arange(steps)[::-1]
    return float(np.sum(np.mean(np.square(predict - target[:, None]) * w, axis=0)))
