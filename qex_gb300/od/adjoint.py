"""Hand-written adjoint of the unrolled 1D SCF (the differentiation configuration).

Losses (``Config3Loss``, ``TrajectoryLoss``), both functions of the
per-iteration total energies and the final mixed density:
  * the differentiation configuration's L = sum_b (E_b - E*_b)^2
    + w sum_b ||n_b - n*_b||^2 dx on the last iteration;
  * the reference's training loss (``qedft/train/od/train.py:250-323``):
    the discounted trajectory MSE of the energies from iteration
    ``ks_iter_to_ignore`` on, over Ne, plus the final-density MSE times dx N,
    over Ne.
The gradient is with respect to the window-MLP parameters: what
``jax.value_and_grad`` over the scanned SCF gives at
``qedft/train/od/trainer.py:139-143``.

Forward: segments of ``checkpoint_every`` iterations, keeping only the input
density of each segment.  Backward: each segment is recomputed from its
checkpoint (one forward launch recording the per-iteration densities) and
swept in reverse with one ``qex_ks1d_adjoint_step`` launch per iteration.
"""

from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from .. import _native as N
from ..xc import resolve
from .engine import Ks1dEngine, PackedBatch, SolveConfig, _convention, _options

_ADJ_SIG = (ctypes.c_int, [ctypes.POINTER(N.Ks1dBatch), ctypes.POINTER(N.Ks1dOptions),
                           ctypes.POINTER(N.XcSpec), ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p])


class Config3Loss:
    """L = sum_b (E_b,T-1 - E*_b)^2 + w sum_b ||n_b - n*_b||^2 dx."""

    def __init__(self, density_weight=0.1):
        self.w = float(density_weight)

    def value(self, energies, final, t_e, t_n, dx_pts, ne, ne_pts):
        de = energies[:, -1] - t_e
        dn = final - t_n
        return float((de * de).sum() + self.w * (dn * dn * dx_pts).sum())

    def grad_density(self, final, t_n, dx_pts, ne_pts, batch_size):
        return 2.0 * self.w * (final - t_n) * dx_pts

    def grad_energy(self, t, energies, t_e, ne):
        T = energies.shape[1]
        return 2.0 * (energies[:, T - 1] - t_e) if t == T - 1 else None


class TrajectoryLoss:
    """The reference's training loss (``qedft/train/od/train.py:296-318`` with
    jax_dft ``losses.trajectory_mse`` / ``mean_square_error``, restated in
    ``qedft/train/od/losses_no_jit.py:8-102``):

      L = mean_b sum_k d^(K-1-k) (E_b,ig+k - E*_b)^2 / Ne
        + mean_b,i (n_b,i - n*_b,i)^2 dx N / Ne,        K = T - ig,

    ig = ``ks_iter_to_ignore``, d = ``discount``; Ne per molecule (the
    reference's datasets hold one Ne), and the density mean taken per molecule
    (sum_i (dn)^2 dx / Ne, averaged over the batch), which is the reference's
    mean over (B, N) times dx N when all molecules share N."""

    def __init__(self, discount=0.9, ks_iter_to_ignore=10):
        self.discount = float(discount)
        self.ignore = int(ks_iter_to_ignore)

    def weights(self, T):
        K = T - self.ignore
        if K < 1:
            raise ValueError("ks_iter_to_ignore leaves no iterations in the loss")
        return self.discount ** np.arange(K - 1, -1, -1, dtype=np.float64)

    def value(self, energies, final, t_e, t_n, dx_pts, ne, ne_pts):
        import torch

        B, T = energies.shape
        w = torch.as_tensor(self.weights(T), device=energies.device)
        de = energies[:, self.ignore:] - t_e[:, None]
        traj = (((de * de) * w[None, :]).sum(dim=1) / ne).sum() / B
        dn = final - t_n
        dens = (dn * dn * dx_pts / ne_pts).sum() / B
        return float(traj + dens)

    def grad_density(self, final, t_n, dx_pts, ne_pts, batch_size):
        return 2.0 * (final - t_n) * dx_pts / ne_pts / batch_size

    def grad_energy(self, t, energies, t_e, ne):
        B, T = energies.shape
        if t < self.ignore:
            return None
        w = self.weights(T)[t - self.ignore]
        return 2.0 * w * (energies[:, t] - t_e) / ne / B


@dataclasses.dataclass
class AdjointResult:
    loss: float
    grad: np.ndarray  # (577,) float64, flat window-MLP parameter order
    energies: np.ndarray  # (B, T)
    final_density: np.ndarray  # packed
    status: np.ndarray


class Ks1dAdjoint:
    def __init__(self, engine: Ks1dEngine | None = None):
        self.engine = engine or Ks1dEngine()
        self.lib = self.engine.lib
        fn = self.lib.qex_ks1d_adjoint_step
        fn.restype, fn.argtypes = _ADJ_SIG
        ws = self.lib.qex_ks1d_adjoint_workspace_size
        ws.restype = ctypes.c_int
        ws.argtypes = [ctypes.POINTER(N.Ks1dOptions), ctypes.c_int32,
                       ctypes.POINTER(ctypes.c_size_t)]

    def forward(self, batch: PackedBatch, xc, cfg: SolveConfig, checkpoint_every: int = 5,
                initial_density=None):
        """The forward half of a ``jax.custom_vjp`` (``fwd``): the unrolled SCF
        with checkpoints.  Returns ((energies (B, T), final mixed density
        (packed)), residuals); the residuals are the checkpointed input
        densities of every ``checkpoint_every``-iteration segment, from which
        ``backward`` recomputes the iterates.  ``initial_density`` (packed)
        defaults to the non-interacting density of v_ext (jax_dft
        ``get_initial_density(..., 'noninteracting')``)."""
        torch = N.require_cuda()
        if cfg.convention != "local" or cfg.num_mixing_iterations != 1:
            raise ValueError("the adjoint covers the local convention with one mixing difference")
        if cfg.density_mse_converge_tolerance > 0:
            raise ValueError("the adjoint differentiates the fixed-iteration SCF "
                             "(density_mse_converge_tolerance <= 0)")
        dev = batch.device
        T = int(cfg.num_iterations)
        B = batch.size
        if initial_density is not None:
            n0 = torch.as_tensor(np.asarray(initial_density, np.float64), device=dev).contiguous()
        else:
            # non-interacting ground state of v_ext
            one = SolveConfig(**{**dataclasses.asdict(cfg), "num_iterations": 1})
            out1 = self.engine.solve(batch, xc, one, records=("external_potential",),
                                     bucketed=False)
            n0, _, _, _ = self.engine.noninteracting(batch, out1["external_potential"],
                                                     cfg.stencil)
        checkpoints = {}
        energies = torch.empty((B, T), dtype=torch.float64, device=dev)
        n = n0
        for t0 in range(0, T, checkpoint_every):
            steps = min(checkpoint_every, T - t0)
            checkpoints[t0] = n
            out = self._segment(batch, xc, cfg, n, t0, steps, ("energy", "final_density"))
            energies[:, t0:t0 + steps] = out["energy"]
            n = out["final_density"].clone()
        residuals = {"batch": batch, "xc": xc, "cfg": cfg, "checkpoints": checkpoints,
                     "checkpoint_every": checkpoint_every, "status": out["status"].clone()}
        return (energies, n), residuals

    def _segment(self, batch, xc, cfg, n_start, t0, steps, records):
        c = SolveConfig(**{**dataclasses.asdict(cfg), "num_iterations": steps,
                           "alpha": cfg.alpha * cfg.alpha_decay ** t0})
        return self.engine.solve(batch, xc, c, records=records, initial_density=n_start,
                                 bucketed=False)

    def backward(self, residuals, cotangents):
        """The backward half of a ``jax.custom_vjp`` (``bwd``): cotangents
        (g_energies (B, T) or None, g_final_density (packed) or None) -> the
        gradient with respect to the window-MLP parameters (flat, 577 FP64),
        by one ``qex_ks1d_adjoint_step`` launch per iteration, each segment's
        iterates recomputed from its checkpoint."""
        torch = N.require_cuda()
        batch, xc, cfg = residuals["batch"], residuals["xc"], residuals["cfg"]
        checkpoints, every = residuals["checkpoints"], residuals["checkpoint_every"]
        functional, params = resolve(xc)
        spec, keep = functional.spec(params, _convention(cfg))
        dev = batch.device
        T = int(cfg.num_iterations)
        B = batch.size
        P = batch.total_points
        g_e, g_n = cotangents
        gnext = (torch.zeros(P, dtype=torch.float64, device=dev) if g_n is None else
                 torch.as_tensor(g_n, dtype=torch.float64, device=dev).clone().contiguous())
        g_e = None if g_e is None else torch.as_tensor(g_e, dtype=torch.float64, device=dev)
        genergy = torch.zeros(B, dtype=torch.float64, device=dev)
        gtheta = torch.zeros((B, N.MLP_NUM_PARAMS), dtype=torch.float64, device=dev)
        gn = torch.empty_like(gnext)
        opts = _options(cfg, batch, False)
        nb = ctypes.c_size_t()
        N.check(self.lib.qex_ks1d_adjoint_workspace_size(ctypes.byref(opts), B, ctypes.byref(nb)),
                "qex_ks1d_adjoint_workspace_size")
        ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        st = torch.zeros(B, dtype=torch.int32, device=dev)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        cb = batch.c_batch()
        for t0 in sorted(checkpoints, reverse=True):
            steps = min(every, T - t0)
            # recompute the segment's per-iteration input densities
            if steps > 1:
                rec = self._segment(batch, xc, cfg, checkpoints[t0], t0, steps - 1,
                                    ("density",))["density"]
                dens_rec = rec  # (steps-1) x packed, molecule-major
            inputs = [checkpoints[t0]]
            for k in range(1, steps):
                x = torch.empty(P, dtype=torch.float64, device=dev)
                for b in range(B):
                    nb_, o_ = int(batch.num_grids_host[b]), int(batch.offsets_host[b])
                    base = (steps - 1) * o_ + (k - 1) * nb_
                    x[o_:o_ + nb_] = dens_rec[base: base + nb_]
                inputs.append(x)
            for k in range(steps - 1, -1, -1):
                t = t0 + k
                if g_e is None:
                    genergy.zero_()
                else:
                    genergy.copy_(g_e[:, t])
                alpha_t = cfg.alpha * cfg.alpha_decay ** t
                rc = self.lib.qex_ks1d_adjoint_step(
                    ctypes.byref(cb), ctypes.byref(opts), ctypes.byref(spec),
                    ctypes.c_void_p(inputs[k].data_ptr()), ctypes.c_void_p(gnext.data_ptr()),
                    ctypes.c_void_p(genergy.data_ptr()), ctypes.c_double(alpha_t),
                    ctypes.c_void_p(gn.data_ptr()), ctypes.c_void_p(gtheta.data_ptr()),
                    ctypes.c_void_p(st.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                    ctypes.c_size_t(ws.numel()), stream)
                N.check(rc, "qex_ks1d_adjoint_step")
                gnext, gn = gn, gnext
        grad = gtheta.sum(dim=0)
        torch.cuda.current_stream().synchronize()
        del keep
        return grad.cpu().numpy()

    def value_and_grad(self, batch: PackedBatch, xc, cfg: SolveConfig, target_energy,
                       target_density, density_weight: float = 0.1,
                       checkpoint_every: int = 5, loss=None,
                       initial_density=None) -> AdjointResult:
        """Loss and gradient; ``loss`` is a ``Config3Loss`` (the default, with
        ``density_weight``) or a ``TrajectoryLoss``.  Reflection symmetry
        (``cfg.enforce_reflection_symmetry``) is differentiated as well.
        ``forward`` then ``backward`` with the loss's cotangents."""
        torch = N.require_cuda()
        if loss is None:
            loss = Config3Loss(density_weight)
        dev = batch.device
        B = batch.size
        dx = torch.as_tensor(np.repeat(np.array([m.grid_spacing for m in batch.molecules]),
                                       batch.num_grids_host), device=dev)
        t_e = torch.as_tensor(np.asarray(target_energy, np.float64), device=dev)
        t_n = torch.as_tensor(np.asarray(target_density, np.float64), device=dev)
        ne_host = np.array([m.num_electrons for m in batch.molecules], dtype=np.float64)
        ne = torch.as_tensor(ne_host, device=dev)
        ne_pts = torch.as_tensor(np.repeat(ne_host, batch.num_grids_host), device=dev)
        (energies, n), res = self.forward(batch, xc, cfg, checkpoint_every, initial_density)
        loss_value = loss.value(energies, n, t_e, t_n, dx, ne, ne_pts)
        T = energies.shape[1]
        g_e = torch.zeros((B, T), dtype=torch.float64, device=dev)
        for t in range(T):
            ge = loss.grad_energy(t, energies, t_e, ne)
            if ge is not None:
                g_e[:, t] = ge
        g_n = loss.grad_density(n, t_n, dx, ne_pts, B).contiguous()
        grad = self.backward(res, (g_e, g_n))
        return AdjointResult(loss=loss_value, grad=grad, energies=energies.cpu().numpy(),
                             final_density=n.cpu().numpy(), status=res["status"].cpu().numpy())


def scf_fwd(xc, batch: PackedBatch, cfg: SolveConfig, checkpoint_every: int = 5,
            initial_density=None, adjoint: Ks1dAdjoint | None = None):
    """``fwd`` of ``jax.custom_vjp`` over the unrolled SCF (the reference
    differentiates ``jax.lax.scan`` at ``qedft/train/od/jit_scf.py:184-211``
    with ``jax.value_and_grad`` at ``qedft/train/od/trainer.py:139-143``):
    ((energies, final density), residuals)."""
    adj = adjoint or Ks1dAdjoint()
    out, res = adj.forward(batch, xc, cfg, checkpoint_every, initial_density)
    res["adjoint"] = adj
    return out, res


def scf_bwd(residuals, cotangents):
    """``bwd`` of ``jax.custom_vjp``: (g_energies, g_final_density) -> the
    parameter gradient (flat window-MLP order, 577 FP64)."""
    return residuals["adjoint"].backward(residuals, cotangents)

