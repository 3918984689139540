"""Launch-plan autotuner of the batched 1D solver.

The batched SCF is one persistent kernel per launch; what is left to choose
per batch shape is the launch plan: split the batch into eigenpair-count runs
launched concurrently (the shared memory per warp scales with K) or launch it
whole, and keep the FP32 solve planes resident in shared memory (fewest
instructions, fewer warps per SM) or stream them through the ring (more warps
per SM), and with streamed planes the tile of the ring: 16, 32 or 64 points
per chunk (more chunks in flight hide more latency; larger chunks take more
shared memory per warp, so fewer warps per SM).  The best plan depends on the
mix of grid sizes and electron counts and on the XC functional, so the tuner
times the candidates on the batch itself (a few SCF iterations each, CUDA
events on the current stream) the first time a batch shape is seen, and
caches the winner.
"""

from __future__ import annotations

import dataclasses

from .. import _native as N

# (bucketed, solve_planes, solve_chunk): solve_planes 0 = the library's
# automatic choice, 1 = resident, 2 = streamed; solve_chunk 0 = the default 32
CANDIDATES = ((True, 2, 32), (True, 2, 16), (True, 2, 64), (True, 1, 0), (False, 2, 32),
              (False, 0, 0))


@dataclasses.dataclass(frozen=True)
class Plan:
    bucketed: bool
    planes: int
    chunk: int = 0


class PlanTuner:
    def __init__(self, trial_iterations: int = 3, candidates=CANDIDATES):
        self.trial_iterations = int(trial_iterations)
        self.candidates = tuple(candidates)
        self.cache: dict = {}
        self.timings: dict = {}

    @staticmethod
    def key(batch, functional_kind, cfg):
        """Shape key: molecules per (N, K) class, XC kind, stencil, convention."""
        import numpy as np

        ng = np.asarray(batch.num_grids_host)
        k = np.asarray([m.num_electrons // 2 + 1 for m in batch.molecules])
        pairs, counts = np.unique(np.stack([ng, k]), axis=1, return_counts=True)
        hist = tuple((int(a), int(b), int(c)) for (a, b), c in zip(pairs.T, counts))
        return (hist, int(functional_kind), int(cfg.stencil), cfg.convention,
                int(cfg.num_mixing_iterations), bool(cfg.enforce_reflection_symmetry))

    def plan(self, engine, batch, xc, cfg, functional_kind) -> Plan:
        key = self.key(batch, functional_kind, cfg)
        hit = self.cache.get(key)
        if hit is not None:
            return hit
        torch = N.require_cuda()
        trial = dataclasses.replace(cfg, num_iterations=min(self.trial_iterations,
                                                            int(cfg.num_iterations)))
        out = engine.allocate_outputs(batch, trial, ("energy",))
        times = {}
        for cand in self.candidates:
            bucketed, planes = cand[0], cand[1]
            chunk = cand[2] if len(cand) > 2 else 0
            if bucketed and len(batch.buckets) <= 1:
                continue
            # one untimed run (kernel attributes, workspace growth), one timed
            engine.solve(batch, xc, trial, out=out, bucketed=bucketed, planes=planes,
                         chunk=chunk, tune=False)
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record()
            engine.solve(batch, xc, trial, out=out, bucketed=bucketed, planes=planes,
                         chunk=chunk, tune=False)
            stop.record()
            stop.synchronize()
            times[(bucketed, planes, chunk)] = start.elapsed_time(stop)
        best = min(times, key=times.get)
        plan = Plan(bucketed=best[0], planes=best[1], chunk=best[2])
        self.cache[key] = plan
        self.timings[key] = times
        return plan
