"""Continuous-batching SCF server (the serving configuration).

Requests arrive over time: 1D Kohn-Sham solves of any grid size and electron
count, and 3D SCF solves (numint LDA + DIIS) of resident molecules.  The
server admits every pending 1D request into a new batch as soon as a launch
slot (a CUDA stream) and device memory are free, so batches launched at
different times run concurrently on the GPU; each request's density,
eigenvectors and mixing history stay in its batch's device workspace until
the solve ends.  A 3D request replays its molecule's captured SCF graph
(``qex_gb300.td.graph.CapturedScf``: integrals, density matrix and DIIS
history resident on the device) on a free stream; a 3D request for a
molecule that is not resident is admitted by building it first (grid, AO
values and integrals on the GPU, then the captured graph), and that set-up is
part of its latency.  The streams split into a 1D share and a 3D share
(``max_inflight3d``), so that neither kind of backlog holds back the other,
and a new 3D molecule is set up one stage per pass of the loop (one molecule
at a time), so that 1D batches launch between its stages.  Admission is
by device memory: a batch is admitted only
while its estimated bytes fit the free HBM the driver reports
(``cudaMemGetInfo``, through ``torch.cuda.mem_get_info``, plus the memory the
allocator caches but does not use) less a safety margin, or, when
``memory_budget_bytes`` is given, while the in-flight batches and resident 3D
graphs stay under that budget.  Latency is arrival -> result on the host.

The reference has no serving layer; it solves one molecule (or one vmap'd
batch of equal-shape molecules) per call (``qedft/train/od/train.py:84-125``),
which is what ``serve_plain`` reproduces: one request at a time.
"""

from __future__ import annotations

import ctypes
import dataclasses
import time
from typing import List, Sequence

import numpy as np

from . import _native as N
from .od.engine import Ks1dEngine, Molecule1D, PackedBatch, SolveConfig, _convention, _options
from .xc import resolve


@dataclasses.dataclass
class Request:
    rid: int
    molecule: Molecule1D | None  # 1D request
    arrival: float  # seconds from the start of the stream
    start: float = float("nan")
    finish: float = float("nan")
    energies: np.ndarray | None = None
    density: np.ndarray | None = None
    status: int = 0
    graph3d: object = None  # 3D request: key of a resident CapturedScf
    e_tot: float | None = None  # 3D: energy at the cycle the stop rule was met (else the last)
    converged3d: bool = False   # 3D: the reference's stop rule (|dE|, |g|) was met

    @property
    def is3d(self):
        return self.graph3d is not None

    @property
    def latency(self):
        return self.finish - self.arrival


@dataclasses.dataclass
class _Launch:
    requests: List[Request]
    batch: PackedBatch | None
    out: dict | None
    host: dict
    workspace: object
    stream: object
    event: object
    nbytes: int
    graph3d: object = None


def config1_requests(arrivals, seed: int = 0, num_grids=513, spacing=0.08) -> List[Request]:
    """H2-like 1D requests of the plain configuration's shape (513 points,
    dx 0.08, unit charges at +-R with R uniform in [0.5, 1.5] bohr)."""
    rng = np.random.default_rng(seed)
    out = []
    for i, t in enumerate(arrivals):
        r = rng.uniform(0.5, 1.5)
        mol = Molecule1D(num_grids=num_grids, grid_spacing=spacing, locations=[-r, r],
                         nuclear_charges=[1.0, 1.0], num_electrons=2)
        out.append(Request(rid=i, molecule=mol, arrival=float(t)))
    return out


def poisson_arrivals(rate: float, duration: float, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n = rng.poisson(rate * duration)
    return np.sort(rng.uniform(0.0, duration, n))


class ScfServer:
    """Continuous batching of 1D SCF requests over a pool of CUDA streams."""

    def __init__(self, xc, cfg: SolveConfig, max_inflight: int = 16, max_batch: int = 512,
                 memory_budget_bytes: int | None = None, engine: Ks1dEngine | None = None,
                 graphs3d: dict | None = None, builder3d=None, max_cycle3d: int = 30,
                 hbm_margin_bytes: int = 2 << 30, max_inflight3d: int | None = None):
        self.torch = N.require_cuda()
        self.xc = xc
        self.cfg = cfg
        self.engine = engine or Ks1dEngine()
        self.lib = self.engine.lib
        self.max_inflight = max_inflight
        self.max_batch = max_batch
        self.budget = memory_budget_bytes
        self.streams = [self.torch.cuda.Stream() for _ in range(max_inflight)]
        # the streams split into a 1D share and a 3D share, so that a 3D
        # backlog (seconds of replays) never holds back the 1D batches and
        # the reverse; without 3D molecules 1D has every stream
        has3d = bool(graphs3d) or builder3d is not None
        if max_inflight3d is None:
            max_inflight3d = max_inflight // 2 if has3d else 0
        if has3d and not 1 <= max_inflight3d < max_inflight:
            raise ValueError("with 3D molecules, 1 <= max_inflight3d < max_inflight")
        self.max_inflight3d = max_inflight3d
        self.functional, self.params = resolve(xc)
        self.spec, self._keep = self.functional.spec(self.params, _convention(cfg))
        # resident 3D molecules (captured SCF graphs) hold their memory throughout
        self.graphs3d = dict(graphs3d or {})
        self.resident = sum(g.nbytes for g in self.graphs3d.values())
        self.busy3d = set()
        self.in_use = 0
        self.launches = 0
        # builder3d(key) -> molecule: how a 3D request for a molecule that is
        # not resident is built (its graph is then captured and kept)
        self.builder3d = builder3d
        self.max_cycle3d = max_cycle3d
        self.margin = hbm_margin_bytes
        self.built3d = 0
        self._building = None  # (key, graph, remaining stages) of a molecule being set up

    def _fits(self, nbytes: int) -> bool:
        """Admission test: the fixed budget when given, else the free HBM."""
        if self.budget is not None:
            return self.in_use + self.resident + nbytes <= self.budget
        free, _ = self.torch.cuda.mem_get_info()
        cached = self.torch.cuda.memory_reserved() - self.torch.cuda.memory_allocated()
        return nbytes <= free + cached - self.margin

    def _ensure3d(self, key):
        """Make the molecule of a 3D request resident (build + capture) if needed."""
        while self._building is not None:  # finish a set-up in progress first
            self._advance_build()
        if key in self.graphs3d:
            return
        self._start_build(key)
        while self._building is not None:
            self._advance_build()

    def _start_build(self, key):
        """First stage of a new molecule's set-up (the builder: grid, AO
        values, integrals); the rest runs one stage per pass of the loop."""
        from .td.graph import CapturedScf

        mol = self.builder3d(key)
        g = CapturedScf.__new__(CapturedScf)
        self._building = (key, g, g.build_stages(mol, max_cycle=self.max_cycle3d))

    def _advance_build(self):
        """One more stage of the molecule being set up (eigensolver autotune,
        warm-up SCF, capture); the molecule is resident after the last."""
        key, g, stages = self._building
        try:
            next(stages)
        except StopIteration:
            self.graphs3d[key] = g
            self.resident += g.nbytes
            self.built3d += 1
            self._building = None
        except BaseException:
            self._building = None  # a failed set-up leaves nothing half-built behind
            raise

    def _bytes_for(self, batch: PackedBatch, opts) -> int:
        nb = ctypes.c_size_t()
        N.check(self.lib.qex_ks1d_workspace_size(ctypes.byref(opts), batch.size, ctypes.byref(nb)),
                "qex_ks1d_workspace_size")
        T = self.cfg.num_iterations
        outputs = batch.size * T * 8 * 2 + batch.total_points * 8 + batch.size * (8 + 16 + 64)
        return nb.value + outputs

    def _launch(self, reqs: Sequence[Request], stream, now: float) -> _Launch:
        torch = self.torch
        with torch.cuda.stream(stream):
            batch = PackedBatch([r.molecule for r in reqs], sort=False)
            opts = _options(self.cfg, batch, False)
            nbytes = self._bytes_for(batch, opts)
            out = self.engine.allocate_outputs(batch, self.cfg, ("energy", "final_density"))
            nb = ctypes.c_size_t()
            self.lib.qex_ks1d_workspace_size(ctypes.byref(opts), batch.size, ctypes.byref(nb))
            ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device="cuda")
            cb = batch.c_batch()
            co = self.engine._c_outputs(out)
            rc = self.lib.qex_ks1d_solve(ctypes.byref(cb), ctypes.byref(opts), ctypes.byref(self.spec),
                                         ctypes.byref(co), ctypes.c_void_p(ws.data_ptr()),
                                         ctypes.c_size_t(ws.numel()),
                                         ctypes.c_void_p(stream.cuda_stream))
            N.check(rc, "qex_ks1d_solve")
            host = {k: torch.empty(out[k].shape, dtype=out[k].dtype, pin_memory=True)
                    for k in ("energy", "final_density", "status")}
            for k, t in host.items():
                t.copy_(out[k], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        self.launches += 1
        for r in reqs:
            r.start = now
        return _Launch(list(reqs), batch, out, host, ws, stream, ev, nbytes)

    def _launch3d(self, req: Request, stream, now: float) -> _Launch:
        torch = self.torch
        g = self.graphs3d[req.graph3d]
        with torch.cuda.stream(stream):
            res = g.replay()
            host = {"energy": torch.empty(res.energies.shape, dtype=torch.float64, pin_memory=True),
                    "status": torch.empty(res.status.shape, dtype=torch.int32, pin_memory=True),
                    "e_tot": torch.empty(1, dtype=torch.float64, pin_memory=True),
                    "state": torch.empty(3, dtype=torch.int32, pin_memory=True)}
            host["energy"].copy_(res.energies, non_blocking=True)
            host["status"].copy_(res.status, non_blocking=True)
            host["e_tot"].copy_(res.e_tot, non_blocking=True)
            host["state"].copy_(res.converged, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        self.busy3d.add(req.graph3d)
        self.launches += 1
        req.start = now
        return _Launch([req], None, None, host, None, stream, ev, 0, graph3d=req.graph3d)

    def _retire(self, launch: _Launch, now: float):
        if launch.graph3d is not None:
            r = launch.requests[0]
            r.finish = now
            r.energies = launch.host["energy"].numpy().copy()
            r.status = int(np.bitwise_or.reduce(launch.host["status"].numpy()))
            r.e_tot = float(launch.host["e_tot"].numpy()[0])
            r.converged3d = bool(launch.host["state"].numpy()[0])
            self.busy3d.discard(launch.graph3d)
            return
        energy = launch.host["energy"].numpy()
        dens = launch.batch.split(launch.host["final_density"].numpy())
        status = launch.host["status"].numpy()
        for i, r in enumerate(launch.requests):
            r.finish = now
            r.energies = energy[i].copy()
            r.density = dens[i].copy()
            r.status = int(status[i])
        self.in_use -= launch.nbytes

    def serve(self, requests: Sequence[Request], realtime: bool = True,
              deadline: float | None = None) -> List[Request]:
        """Serve ``requests`` (sorted by arrival) and return them.

        With ``deadline`` (seconds from the start), nothing new is launched
        after it: the work in flight completes and the requests still waiting
        are returned unserved (``finish`` NaN), as a load test of an
        overloaded server reports them.

        Pending 1D requests wait in one FIFO, pending 3D requests in one FIFO
        per molecule (a molecule's graph replays one request at a time), so
        each pass of the loop costs O(batch + molecules) however long the
        backlog grows."""
        import collections

        reqs = sorted(requests, key=lambda r: r.arrival)
        pending1d = collections.deque()
        pending3d = collections.OrderedDict()  # molecule -> deque of requests
        inflight: List[_Launch] = []
        free = list(self.streams[self.max_inflight3d:])
        free3d = list(self.streams[: self.max_inflight3d])
        nxt = 0
        t0 = time.perf_counter()
        done = 0
        while done < len(reqs):
            now = time.perf_counter() - t0
            if deadline is not None and now > deadline:
                for L in inflight:
                    L.event.synchronize()
                    self._retire(L, time.perf_counter() - t0)
                break
            if (not realtime and not pending1d and not pending3d and not inflight
                    and nxt < len(reqs)):
                now = reqs[nxt].arrival
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                r = reqs[nxt]
                if r.is3d:
                    pending3d.setdefault(r.graph3d, collections.deque()).append(r)
                else:
                    pending1d.append(r)
                nxt += 1
            for L in list(inflight):
                if L.event.query():
                    self._retire(L, time.perf_counter() - t0)
                    done += len(L.requests)
                    inflight.remove(L)
                    (free3d if L.graph3d is not None else free).append(L.stream)
            self._launch1d(pending1d, free, inflight, now)
            # A new 3D molecule is set up one stage per pass (each stage waits
            # for the GPU), so the 1D batches that arrive meanwhile launch
            # between its stages; one molecule is set up at a time.
            if self._building is not None:
                self._advance_build()
                now = time.perf_counter() - t0
            # 3D requests: a replay of the molecule's graph on a free 3D stream
            # (one replay of a graph at a time: its results are static tensors);
            # the molecule whose oldest request arrived first goes first.
            if pending3d and free3d:
                order = sorted((q[0].arrival, k) for k, q in pending3d.items()
                               if k not in self.busy3d)
                for _, key in order:
                    if not free3d:
                        break
                    if key not in self.graphs3d:
                        if self.builder3d is None:
                            raise KeyError(f"3D molecule {key!r} is not resident")
                        if self._building is None:
                            self._start_build(key)  # set-up inside this request's latency
                            now = time.perf_counter() - t0
                        continue
                    q = pending3d[key]
                    r = q.popleft()
                    if not q:
                        del pending3d[key]
                    inflight.append(self._launch3d(r, free3d.pop(), now))
            if realtime:
                time.sleep(0.0002)
        return reqs

    def _launch1d(self, pending1d, free, inflight, now):
        """Launch the pending 1D requests in batches while streams are free."""
        while free and pending1d:
            take = [pending1d[i] for i in range(min(self.max_batch, len(pending1d)))]
            # admission by device memory: halve the batch until it fits; a
            # single request that does not fit waits for in-flight batches
            # to finish (or runs alone on an idle GPU)
            while len(take) > 1 and not self._fits(self._estimate(take)):
                take = take[: len(take) // 2]
            if not self._fits(self._estimate(take)) and inflight:
                break
            L = self._launch(take, free.pop(), now)
            self.in_use += L.nbytes
            inflight.append(L)
            for _ in range(len(take)):
                pending1d.popleft()

    def _estimate(self, reqs: Sequence[Request]) -> int:
        n = sum(r.molecule.num_grids for r in reqs)
        nmax = max(r.molecule.num_grids for r in reqs)
        kmax = max(r.molecule.num_electrons // 2 + 1 for r in reqs)
        slots = min(self.cfg.num_mixing_iterations, self.cfg.num_iterations)
        # FP64 vectors + the FP32 solve planes of one molecule (ks1d.cu workspace)
        per = (9 + slots + kmax + 2) * nmax * 8 + -(-nmax // 16) * 16 * kmax * 12
        return len(reqs) * per + len(reqs) * self.cfg.num_iterations * 16 + n * 8


def serve_plain(xc, cfg: SolveConfig, requests: Sequence[Request],
                engine: Ks1dEngine | None = None, molecules3d: dict | None = None,
                max_cycle: int = 30) -> List[Request]:
    """One request at a time, in arrival order (the reference's calling pattern):
    1D requests through the engine, 3D requests through ``td.scf.run_scf`` (kernel
    launches from the host, no graph) on the molecule in ``molecules3d``."""
    torch = N.require_cuda()
    engine = engine or Ks1dEngine()
    reqs = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    for r in reqs:
        now = time.perf_counter() - t0
        if now < r.arrival:
            time.sleep(r.arrival - now)
        r.start = time.perf_counter() - t0
        if r.is3d:
            from .td.scf import run_scf

            res = run_scf(molecules3d[r.graph3d], max_cycle)
            r.energies = res.energies.cpu().numpy()
            r.status = int(np.bitwise_or.reduce(res.status.cpu().numpy()))
            r.e_tot = float(res.e_tot.cpu().numpy()[0])
            r.converged3d = bool(res.converged.cpu().numpy()[0])
            r.finish = time.perf_counter() - t0
            continue
        batch = PackedBatch([r.molecule], sort=False)
        out = engine.solve(batch, xc, cfg, records=("energy", "final_density"))
        energy = out["energy"].cpu().numpy()
        r.density = out["final_density"].cpu().numpy()
        r.status = int(out["status"].cpu().numpy()[0])
        r.energies = energy[0]
        r.finish = time.perf_counter() - t0
    return reqs


def mixed_requests(arrivals, keys3d: Sequence, frac3d: float = 0.2, seed: int = 0,
                   num_grids=513, spacing=0.08) -> List[Request]:
    """Config-5 stream: a fraction ``frac3d`` of 3D requests (uniform over the
    resident molecules ``keys3d``), the rest config-1-shaped 1D requests."""
    rng = np.random.default_rng(seed)
    out = []
    for i, t in enumerate(arrivals):
        if keys3d and rng.uniform() < frac3d:
            out.append(Request(rid=i, molecule=None, arrival=float(t),
                               graph3d=keys3d[int(rng.integers(len(keys3d)))]))
        else:
            r = rng.uniform(0.5, 1.5)
            mol = Molecule1D(num_grids=num_grids, grid_spacing=spacing, locations=[-r, r],
                             nuclear_charges=[1.0, 1.0], num_electrons=2)
            out.append(Request(rid=i, molecule=mol, arrival=float(t)))
    return out


def latency_summary(reqs: Sequence[Request], duration: float | None = None) -> dict:
    out = _summary(reqs, duration)
    if any(r.is3d for r in reqs) and not all(r.is3d for r in reqs):
        span = out.get("span_s")
        out["1d"] = _summary([r for r in reqs if not r.is3d], span)
        out["3d"] = _summary([r for r in reqs if r.is3d], span)
    return out


def _summary(reqs: Sequence[Request], duration: float | None = None) -> dict:
    unserved = sum(1 for r in reqs if not np.isfinite(r.finish))
    reqs = [r for r in reqs if np.isfinite(r.finish)]
    if not reqs:
        return {"requests": 0, "unserved": unserved}
    lat = np.array([r.latency for r in reqs])
    span = duration if duration else (max(r.finish for r in reqs) - min(r.arrival for r in reqs))
    # 1D: |E_T - E_T-1| < 1e-8 Ha with the status clear; 3D: the reference's
    # stop rule (|dE| < conv_tol and |g| < conv_tol_grad) met on the device
    conv = [r for r in reqs if (r.converged3d if r.is3d else (
        r.energies is not None and abs(r.energies[-1] - r.energies[-2]) < 1e-8))
        and (r.status & 0xFFFF) == 0]
    return {
        "requests": len(reqs),
        "unserved": unserved,
        "converged": len(conv),
        "solves_per_s": len(reqs) / span if span > 0 else float("nan"),
        "converged_solves_per_s": len(conv) / span if span > 0 else float("nan"),
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "mean_ms": float(lat.mean() * 1e3),
        "span_s": float(span),
    }
