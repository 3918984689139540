"""Hand-written adjoint of the unrolled 1D SCF (the differentiation configuration).

Loss (per batch): L = sum_b (E_b - E*_b)^2 + w sum_b ||n_b - n*_b||^2 dx, with
E the last iteration's total energy and n the final mixed density; gradient
with respect to the window-MLP parameters (what ``jax.value_and_grad`` over
the scanned SCF gives at ``qedft/train/od/trainer.py:139-143``, with the loss
of ``qedft/train/od/train.py:250-323`` replaced by this one).

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

    def value_and_grad(self, batch: PackedBatch, xc, cfg: SolveConfig, target_energy,
                       target_density, density_weight: float = 0.1,
                       checkpoint_every: int = 5) -> AdjointResult:
        torch = N.require_cuda()
        if cfg.convention != "local" or cfg.num_mixing_iterations != 1:
            raise ValueError("the adjoint covers the local convention with one mixing difference")
        functional, params = resolve(xc)
        spec, keep = functional.spec(params, _convention(cfg))
        dev = batch.device
        T = int(cfg.num_iterations)
        B = batch.size
        dx = torch.as_tensor(np.repeat(np.array([m.grid_spacing for m in batch.molecules]),
                                       batch.num_grids_host), device=dev)
        t_e = torch.as_tensor(np.asarray(target_energy, np.float64), device=dev)
        t_n = torch.as_tensor(np.asarray(target_density, np.float64), device=dev)

        # initial density: non-interacting ground state of v_ext
        one = SolveConfig(**{**dataclasses.asdict(cfg), "num_iterations": 1})
        out1 = self.engine.solve(batch, xc, one, records=("external_potential",), bucketed=False)
        n0, _, _, _ = self.engine.noninteracting(batch, out1["external_potential"], cfg.stencil)

        def segment(n_start, t0, steps, records):
            c = SolveConfig(**{**dataclasses.asdict(cfg), "num_iterations": steps,
                               "alpha": cfg.alpha * cfg.alpha_decay ** t0})
            return self.engine.solve(batch, xc, c, records=records, initial_density=n_start,
                                     bucketed=False)

        # ---- forward with checkpoints
        checkpoints = {}
        energies = torch.empty((B, T), dtype=torch.float64, device=dev)
        n = n0
        for t0 in range(0, T, checkpoint_every):
            steps = min(checkpoint_every, T - t0)
            checkpoints[t0] = n
            out = segment(n, t0, steps, ("energy", "final_density"))
            energies[:, t0:t0 + steps] = out["energy"]
            n = out["final_density"].clone()
        status = out["status"].clone()
        e_last = energies[:, T - 1]
        de = e_last - t_e
        dn = n - t_n
        loss = float((de * de).sum() + density_weight * (dn * dn * dx).sum())

        # ---- backward
        gnext = (2.0 * density_weight * dn * dx).contiguous()
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
        P = batch.total_points
        for t0 in sorted(checkpoints, reverse=True):
            steps = min(checkpoint_every, T - t0)
            # recompute the segment's per-iteration input densities
            if steps > 1:
                rec = segment(checkpoints[t0], t0, steps - 1, ("density",))["density"]
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
                genergy.zero_()
                if t == T - 1:
                    genergy.copy_(2.0 * de)
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
        return AdjointResult(loss=loss, grad=grad.cpu().numpy(), energies=energies.cpu().numpy(),
                             final_density=n.cpu().numpy(), status=status.cpu().numpy())
