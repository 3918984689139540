"""CUDA-graph capture of the fixed-cycle 3D SCF.

``run_scf`` issues ~10 kernels per cycle from the host and never waits on the
GPU (occupations, DIIS and the eigensolve stay on the device), so the whole
``max_cycle`` loop can be captured once per molecule and replayed: a replay
costs one graph launch instead of ~300 kernel launches and their Python
overhead.  The captured graph reads the molecule's integrals from static
device tensors (resident between requests) and writes static result tensors.
The electron count and the nuclear repulsion are captured constants, so a
graph belongs to one molecule.
"""

from __future__ import annotations

import dataclasses

from .. import _native as N
from .scf import ScfResult, run_scf


@dataclasses.dataclass
class DeviceMolecule3D:
    """The inputs ``run_scf`` reads, as device tensors."""

    ao: object
    weights: object
    s1e: object
    h1e: object
    eri_factors: object
    nelectron: int
    energy_nuc: float

    @classmethod
    def from_host(cls, mol):
        torch = N.require_cuda()

        def dev(a):
            return torch.as_tensor(a, dtype=torch.float64, device="cuda").contiguous()

        return cls(dev(mol.ao), dev(mol.weights), dev(mol.s1e), dev(mol.h1e),
                   dev(mol.eri_factors), int(mol.nelectron), float(mol.energy_nuc))

    @property
    def nao(self):
        return int(self.s1e.shape[0])

    def nbytes(self):
        return sum(t.numel() * t.element_size()
                   for t in (self.ao, self.weights, self.s1e, self.h1e, self.eri_factors))


class CapturedScf:
    """One molecule's ``run_scf(max_cycle)`` captured as a CUDA graph."""

    def __init__(self, mol, max_cycle: int = 30, xc="LDA", tune_eigh: bool = True):
        for _ in self.build_stages(mol, max_cycle, xc, tune_eigh):
            pass

    def build_stages(self, mol, max_cycle: int = 30, xc="LDA", tune_eigh: bool = True):
        """The set-up as a generator: it yields between its stages (the
        eigensolver autotune, the warm-up SCF, the capture), each of which
        waits for the GPU, so that a caller such as the server can launch
        other work between them.  Exhausting it leaves the object ready."""
        torch = N.require_cuda()
        self.max_cycle = max_cycle
        self.mol = mol if isinstance(mol, DeviceMolecule3D) else DeviceMolecule3D.from_host(mol)
        if tune_eigh:
            # the eigensolver path for this basis size, timed on the core Hamiltonian
            from .eigh import tune_path

            self.eigh_path = tune_path(self.mol.h1e, self.mol.s1e)
            yield
        before = torch.cuda.memory_allocated()
        # warm-up outside the capture: kernel attributes, allocator pools
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            run_scf(self.mol, max_cycle, xc=xc)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        yield
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.result: ScfResult = run_scf(self.mol, max_cycle, xc=xc)
        torch.cuda.synchronize()
        # device bytes held while resident: inputs + the graph's private pool
        self.nbytes = self.mol.nbytes() + max(torch.cuda.memory_allocated() - before, 0)

    def replay(self) -> ScfResult:
        """Run the captured SCF on the current stream; results are static tensors."""
        self.graph.replay()
        return self.result
