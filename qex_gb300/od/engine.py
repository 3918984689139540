"""Batched 1D Kohn-Sham engine: packs molecules of uneven grid size and
electron count into the device layout of ``include/qex_ks1d.h`` and calls the
CUDA kernels (one launch per batch solve).

Device memory and streams come from PyTorch; all arithmetic is in the CUDA
library.  Reference behaviour: ``jax.vmap`` of the per-molecule SCF at
``qedft/train/od/train.py:84-125`` (which needs equal grids and one electron
count), generalised to ragged batches.
"""

from __future__ import annotations

import ctypes
import dataclasses
from typing import Sequence

import numpy as np

from .. import _native as N
from ..xc import resolve
from . import utils


@dataclasses.dataclass
class Molecule1D:
    """One 1D system: uniform grid x_i = grid_start + i * grid_spacing."""

    num_grids: int
    grid_spacing: float
    locations: np.ndarray
    nuclear_charges: np.ndarray
    num_electrons: int
    grid_start: float | None = None  # default: centred grid
    initial_density: np.ndarray | None = None
    external_potential: np.ndarray | None = None

    def __post_init__(self):
        self.locations = np.atleast_1d(np.asarray(self.locations, dtype=np.float64))
        self.nuclear_charges = np.atleast_1d(np.asarray(self.nuclear_charges, dtype=np.float64))
        if self.grid_start is None:
            self.grid_start = -0.5 * (self.num_grids - 1) * self.grid_spacing

    @classmethod
    def from_grids(cls, grids, locations, nuclear_charges, num_electrons, **kw):
        grids = np.asarray(grids, dtype=np.float64)
        return cls(num_grids=grids.size, grid_spacing=utils.get_dx(grids), grid_start=float(grids[0]),
                   locations=locations, nuclear_charges=nuclear_charges,
                   num_electrons=int(num_electrons), **kw)

    @property
    def grids(self):
        return self.grid_start + np.arange(self.num_grids) * self.grid_spacing

    @property
    def num_eigenpairs(self):
        return self.num_electrons // 2 + 1


@dataclasses.dataclass
class SolveConfig:
    num_iterations: int = 25
    alpha: float = 0.5
    alpha_decay: float = 0.9
    num_mixing_iterations: int = 1
    density_mse_converge_tolerance: float = -1.0
    enforce_reflection_symmetry: bool = False
    convergence_rule: str = "jit"  # "jit" (scan) or "python" (loop)
    convention: str = "amplitude"  # "amplitude" (qedft) or "local" (jax_dft)
    stencil: int = 5
    interaction: object = utils.exponential_coulomb


RECORD_ALL = ("energy", "gap", "converged", "density", "hartree_potential", "xc_potential",
              "xc_energy_density", "final_density", "external_potential")
RECORD_SUMMARY = ("energy", "gap", "converged", "final_density")


class PackedBatch:
    """Device-resident descriptors of a batch (reusable across solves)."""

    def __init__(self, molecules: Sequence[Molecule1D], device=None, sort=True):
        torch = N.require_cuda()
        self.molecules = list(molecules)
        B = len(self.molecules)
        self.size = B
        ng = np.array([m.num_grids for m in self.molecules], dtype=np.int32)
        off = np.zeros(B, dtype=np.int64)
        if B:
            off[1:] = np.cumsum(ng[:-1].astype(np.int64))
        self.total_points = int(ng.sum()) if B else 0
        self.num_grids_host = ng
        self.offsets_host = off
        self.max_num_grids = int(ng.max()) if B else 5
        ne = np.array([m.num_electrons for m in self.molecules], dtype=np.int32)
        self.num_electrons_host = ne
        self.max_num_electrons = int(ne.max()) if B else 1
        self.max_nuclei = max([m.locations.size for m in self.molecules] + [1])
        loc = np.zeros((B, self.max_nuclei))
        chg = np.zeros((B, self.max_nuclei))
        nn = np.zeros(B, dtype=np.int32)
        for i, m in enumerate(self.molecules):
            k = m.locations.size
            if m.nuclear_charges.size != k:
                raise ValueError("locations and nuclear_charges differ in length")
            loc[i, :k] = m.locations
            chg[i, :k] = m.nuclear_charges
            nn[i] = k
        start = np.array([m.grid_start for m in self.molecules], dtype=np.float64)
        dx = np.array([m.grid_spacing for m in self.molecules], dtype=np.float64)
        kk = ne // 2 + 1
        if sort and B:
            # eigenpair count first (it sizes shared memory), then grid size
            order = np.lexsort((-ng.astype(np.int64), -kk)).astype(np.int32)
        else:
            order = np.arange(B, dtype=np.int32)
        self.order_host = order
        # contiguous runs of equal eigenpair count in processing order
        self.buckets = []
        if sort and B:
            ks = kk[order]
            first = 0
            for i in range(1, B + 1):
                if i == B or ks[i] != ks[first]:
                    sel = order[first:i]
                    self.buckets.append((first, i - first, int(ne[sel].max()), int(ng[sel].max())))
                    first = i
        dev = torch.device("cuda") if device is None else torch.device(device)
        self.device = dev
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), device=dev).to(dt)
        self.num_grids = t(ng, torch.int32)
        self.offsets = t(off, torch.int64)
        self.grid_start = t(start, torch.float64)
        self.grid_spacing = t(dx, torch.float64)
        assert self.grid_start.numel() == B and self.grid_spacing.numel() == B
        self.num_electrons = t(ne, torch.int32)
        self.num_nuclei = t(nn, torch.int32)
        self.locations = t(loc.reshape(-1), torch.float64)
        self.nuclear_charges = t(chg.reshape(-1), torch.float64)
        self.order = t(order, torch.int32)
        self.initial_density = None
        if B and all(m.initial_density is not None for m in self.molecules):
            self.initial_density = t(np.concatenate([np.asarray(m.initial_density, np.float64)
                                                     for m in self.molecules]), torch.float64)
        elif any(m.initial_density is not None for m in self.molecules):
            raise ValueError("give an initial density for every molecule or for none")
        self.external_potential = None
        if B and all(m.external_potential is not None for m in self.molecules):
            self.external_potential = t(np.concatenate(
                [np.asarray(m.external_potential, np.float64) for m in self.molecules]), torch.float64)

    def c_batch(self, initial_density=None, external_potential=None, start=0,
                count=None) -> N.Ks1dBatch:
        b = N.Ks1dBatch()
        b.num_molecules = self.size if count is None else count
        b.num_grids = N.ptr(self.num_grids)
        b.grid_offsets = N.ptr(self.offsets)
        b.grid_start = N.ptr(self.grid_start)
        b.grid_spacing = N.ptr(self.grid_spacing)
        b.num_electrons = N.ptr(self.num_electrons)
        b.num_nuclei = N.ptr(self.num_nuclei)
        b.locations = N.ptr(self.locations)
        b.nuclear_charges = N.ptr(self.nuclear_charges)
        dens = initial_density if initial_density is not None else self.initial_density
        vext = external_potential if external_potential is not None else self.external_potential
        b.initial_density = N.ptr(dens)
        b.external_potential = N.ptr(vext)
        b.order = N.ptr(self.order) + 4 * start if self.size else None
        return b

    def split(self, packed, per_iteration=0):
        """Split a packed (host) array into per-molecule arrays."""
        out = []
        for i in range(self.size):
            n, o = int(self.num_grids_host[i]), int(self.offsets_host[i])
            if per_iteration:
                out.append(packed[per_iteration * o: per_iteration * (o + n)].reshape(per_iteration, n))
            else:
                out.append(packed[o: o + n])
        return out


def _options(cfg: SolveConfig, batch: PackedBatch, vext_given: bool) -> N.Ks1dOptions:
    o = N.Ks1dOptions()
    o.stencil = int(cfg.stencil)
    kind, a, b = utils.interaction_descriptor(cfg.interaction)
    o.interaction = kind
    o.interaction_a, o.interaction_b = a, b
    o.num_iterations = int(cfg.num_iterations)
    o.alpha = float(cfg.alpha)
    o.alpha_decay = float(cfg.alpha_decay)
    o.num_mixing_iterations = int(cfg.num_mixing_iterations)
    o.density_mse_converge_tolerance = float(cfg.density_mse_converge_tolerance)
    o.convergence_rule = {"jit": 0, "python": 1}[cfg.convergence_rule]
    o.enforce_reflection_symmetry = int(bool(cfg.enforce_reflection_symmetry))
    o.external_potential_given = int(vext_given)
    o.max_num_grids = max(batch.max_num_grids, 5)
    o.max_num_electrons = max(batch.max_num_electrons, 1)
    o.max_nuclei = batch.max_nuclei
    return o


def _convention(cfg: SolveConfig) -> int:
    return {"amplitude": N.QEX_XC_AMPLITUDE, "local": N.QEX_XC_LOCAL}[cfg.convention]


class Workspace:
    """Grow-only device workspace (one per engine)."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int):
        torch = N.require_cuda()
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device="cuda")
        return self.buf


class Ks1dEngine:
    """Owns a workspace and runs batched solves on the current torch stream.

    With ``autotune`` the launch plan (eigenpair-count runs or one launch,
    resident or streamed FP32 solve planes) of each new batch shape is chosen
    by timing the candidates on the batch (``qex_gb300.od.autotune``)."""

    def __init__(self, autotune: bool = False):
        self.lib = N.load()
        self.workspace = Workspace()
        self.last_launches = 0
        self.tuner = None
        if autotune:
            from .autotune import PlanTuner

            self.tuner = PlanTuner()

    def _stream(self):
        torch = N.require_cuda()
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def allocate_outputs(self, batch: PackedBatch, cfg: SolveConfig, records=RECORD_ALL):
        torch = N.require_cuda()
        B, T, P = batch.size, int(cfg.num_iterations), batch.total_points
        f64 = dict(dtype=torch.float64, device=batch.device)
        out = {}
        if "energy" in records:
            out["energy"] = torch.empty((B, T), **f64)
        if "gap" in records:
            out["gap"] = torch.empty((B, T), **f64)
        if "converged" in records:
            out["converged"] = torch.empty((B, T), dtype=torch.uint8, device=batch.device)
        for k in ("density", "hartree_potential", "xc_potential", "xc_energy_density"):
            if k in records:
                out[k] = torch.empty((T * P,), **f64)
        if "final_density" in records:
            out["final_density"] = torch.empty((P,), **f64)
        if "external_potential" in records:
            out["external_potential"] = torch.empty((P,), **f64)
        out["status"] = torch.zeros((B,), dtype=torch.int32, device=batch.device)
        out["iterations_run"] = torch.zeros((B,), dtype=torch.int32, device=batch.device)
        out["stats"] = torch.zeros((B, 8), dtype=torch.int32, device=batch.device)
        out["phase_cycles"] = torch.zeros((B, 16), dtype=torch.int64, device=batch.device)
        return out

    @staticmethod
    def _c_outputs(out) -> N.Ks1dOutputs:
        o = N.Ks1dOutputs()
        o.total_energy = N.ptr(out.get("energy"))
        o.gap = N.ptr(out.get("gap"))
        o.converged = N.ptr(out.get("converged"))
        o.density = N.ptr(out.get("density"))
        o.hartree_potential = N.ptr(out.get("hartree_potential"))
        o.xc_potential = N.ptr(out.get("xc_potential"))
        o.xc_energy_density = N.ptr(out.get("xc_energy_density"))
        o.final_density = N.ptr(out.get("final_density"))
        o.external_potential_out = N.ptr(out.get("external_potential"))
        o.status = N.ptr(out.get("status"))
        o.iterations_run = N.ptr(out.get("iterations_run"))
        o.stats = N.ptr(out.get("stats"))
        o.phase_cycles = N.ptr(out.get("phase_cycles"))
        return o

    def solve(self, batch: PackedBatch, xc, cfg: SolveConfig, records=RECORD_ALL, out=None,
              initial_density=None, bucketed=True, planes=None, tune=True, defer_ksr=True,
              chunk=None):
        """Run the full SCF for every molecule of ``batch``.

        With ``bucketed`` the batch is split into runs of equal eigenpair count
        (shared memory per warp scales with it), launched concurrently on
        forked streams; otherwise one launch covers the whole batch.
        ``planes`` overrides the placement of the FP32 solve planes
        (``qex_ks1d_options.solve_planes``: 1 resident, 2 streamed) and
        ``chunk`` the points per chunk of the streamed planes' ring
        (``qex_ks1d_options.solve_chunk``: 16, 32 or 64).
        ``defer_ksr``: with a KSR functional, size the workspace so that the
        network's energies on the output densities run as one batched launch
        after the SCF (``qex_ks1d_workspace_size_xc``).
        """
        torch = N.require_cuda()
        functional, params = resolve(xc)
        if self.tuner is not None and tune and planes is None and bucketed:
            plan = self.tuner.plan(self, batch, xc, cfg, functional.kind)
            bucketed, planes, chunk = plan.bucketed, plan.planes, plan.chunk
        vext_given = batch.external_potential is not None
        spec, keep = functional.spec(params, _convention(cfg))
        if out is None:
            out = self.allocate_outputs(batch, cfg, records)
        co = self._c_outputs(out)
        parts = batch.buckets if (bucketed and len(batch.buckets) > 1) else [
            (0, batch.size, batch.max_num_electrons, batch.max_num_grids)]
        plans = []
        total = 0
        # concurrent launches share the SMs: past one molecule per SM, stream
        # the FP32 solve planes (small shared-memory footprint, more warps per SM)
        sms = torch.cuda.get_device_properties(batch.device).multi_processor_count
        if planes is None:
            planes = 2 if (len(parts) > 1 and batch.size > sms) else 0
        for start, count, ne_max, ng_max in parts:
            opts = _options(cfg, batch, vext_given)
            opts.max_num_electrons = max(ne_max, 1)
            opts.max_num_grids = max(ng_max, 5)
            opts.solve_planes = planes
            opts.solve_chunk = int(chunk or 0)
            nbytes = ctypes.c_size_t()
            if defer_ksr or functional.kind in (N.QEX_XC_LOCAL_MLP, N.QEX_XC_GLOBAL_MLP):
                N.check(self.lib.qex_ks1d_workspace_size_xc(ctypes.byref(opts), ctypes.byref(spec),
                                                            count, ctypes.byref(nbytes)),
                        "qex_ks1d_workspace_size_xc")
            else:
                N.check(self.lib.qex_ks1d_workspace_size(ctypes.byref(opts), count,
                                                         ctypes.byref(nbytes)),
                        "qex_ks1d_workspace_size")
            aligned = (nbytes.value + 255) // 256 * 256
            plans.append((start, count, opts, total, aligned))
            total += aligned
        ws = self.workspace.get(total)
        base = ws.data_ptr()
        cur = torch.cuda.current_stream()
        launches = 0
        if len(plans) == 1:
            streams = [cur]
        else:
            streams = self._streams(len(plans))
            ev = torch.cuda.Event()
            ev.record(cur)
            for st in streams:
                st.wait_event(ev)
        for (start, count, opts, off, nb), st in zip(plans, streams):
            cb = batch.c_batch(initial_density=initial_density, start=start, count=count)
            rc = self.lib.qex_ks1d_solve(ctypes.byref(cb), ctypes.byref(opts), ctypes.byref(spec),
                                         ctypes.byref(co), ctypes.c_void_p(base + off),
                                         ctypes.c_size_t(nb), ctypes.c_void_p(st.cuda_stream))
            N.check(rc, "qex_ks1d_solve")
            launches += self.lib.qex_last_launch_count()
        if len(plans) > 1:
            for st in streams:
                e = torch.cuda.Event()
                e.record(st)
                cur.wait_event(e)
            ws.record_stream(cur)
        self.last_launches = launches
        del keep
        return out

    def _streams(self, n):
        torch = N.require_cuda()
        pool = getattr(self, "_stream_pool", [])
        while len(pool) < n:
            pool.append(torch.cuda.Stream())
        self._stream_pool = pool
        return pool[:n]

    def iteration(self, batch: PackedBatch, xc, cfg: SolveConfig, density, external_potential):
        """One KS iteration per molecule (unmixed output), records of length 1."""
        functional, params = resolve(xc)
        opts = _options(cfg, batch, True)
        opts.num_iterations = 1
        spec, keep = functional.spec(params, _convention(cfg))
        c1 = SolveConfig(**{**dataclasses.asdict(cfg), "num_iterations": 1})
        out = self.allocate_outputs(batch, c1, ("energy", "gap", "density", "hartree_potential",
                                                "xc_potential", "xc_energy_density"))
        nbytes = ctypes.c_size_t()
        N.check(self.lib.qex_ks1d_workspace_size_xc(ctypes.byref(opts), ctypes.byref(spec),
                                                    batch.size, ctypes.byref(nbytes)),
                "qex_ks1d_workspace_size_xc")
        ws = self.workspace.get(nbytes.value)
        cb = batch.c_batch(external_potential=external_potential)
        co = self._c_outputs(out)
        rc = self.lib.qex_ks1d_iteration(ctypes.byref(cb), ctypes.byref(opts), ctypes.byref(spec),
                                         ctypes.c_void_p(density.data_ptr()), ctypes.byref(co),
                                         ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                         self._stream())
        N.check(rc, "qex_ks1d_iteration")
        self.last_launches = self.lib.qex_last_launch_count()
        del keep
        return out

    def noninteracting(self, batch: PackedBatch, potential, stencil=5):
        torch = N.require_cuda()
        cfg = SolveConfig(num_iterations=1, stencil=stencil)
        opts = _options(cfg, batch, True)
        nbytes = ctypes.c_size_t()
        N.check(self.lib.qex_ks1d_workspace_size(ctypes.byref(opts), batch.size, ctypes.byref(nbytes)),
                "qex_ks1d_workspace_size")
        ws = self.workspace.get(nbytes.value)
        dens = torch.empty((batch.total_points,), dtype=torch.float64, device=batch.device)
        tee = torch.empty((batch.size,), dtype=torch.float64, device=batch.device)
        gap = torch.empty((batch.size,), dtype=torch.float64, device=batch.device)
        status = torch.zeros((batch.size,), dtype=torch.int32, device=batch.device)
        cb = batch.c_batch()
        rc = self.lib.qex_ks1d_noninteracting(
            ctypes.byref(cb), ctypes.byref(opts), ctypes.c_void_p(potential.data_ptr()),
            ctypes.c_void_p(dens.data_ptr()), ctypes.c_void_p(tee.data_ptr()),
            ctypes.c_void_p(gap.data_ptr()), ctypes.c_void_p(status.data_ptr()),
            ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()), self._stream())
        N.check(rc, "qex_ks1d_noninteracting")
        self.last_launches = self.lib.qex_last_launch_count()
        return dens, tee, gap, status


_default_engine = None


def default_engine() -> Ks1dEngine:
    global _default_engine
    if _default_engine is None:
        _default_engine = Ks1dEngine()
    return _default_engine
