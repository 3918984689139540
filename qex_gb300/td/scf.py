"""3D fixed-cycle Kohn-Sham SCF on the GPU.

Mirrors the jit-able padded loop ``qedft/train/td/scf_functions_masked.py:907-967``
(fock = h1e + vhf; DIIS from cycle ``diis_start_cycle``; generalized eigh;
aufbau occupations; density matrix; vhf = J + Vxc; energy) with
``get_occ`` (:176-186), ``make_rdm1`` (``qedft/train/td/hf.py:303-308``), the
CDIIS of ``qedft/train/td/jax_diis.py:10-134`` and the energy of :162-166.
Every step runs on the device; the host only sequences the kernels.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from .. import _native as N
from . import _lib
from .eigh import generalized_eigh
from .numint import _dev, nr_rks


def get_occ(nelectron, mo_energy):
    """2 electrons in each of the lowest Ne/2 orbitals (ties by index)."""
    torch = N.require_cuda()
    mo_energy = _dev(mo_energy, torch.float64)
    order = torch.sort(mo_energy, stable=True).indices
    occ_sorted = (torch.arange(mo_energy.shape[-1], device="cuda") < nelectron // 2).to(torch.float64) * 2.0
    occ = torch.empty_like(occ_sorted)
    occ[order] = occ_sorted
    return occ


def make_rdm1(mo_coeff, mo_occ):
    """D = C diag(occ) C^T (batched when C is (batch, n, n))."""
    torch = N.require_cuda()
    L = _lib.lib()
    C = _dev(mo_coeff, torch.float64)
    occ = _dev(mo_occ, torch.float64)
    single = C.dim() == 2
    if single:
        C, occ = C[None], occ[None]
    batch, n, _ = C.shape
    D = torch.empty_like(C)
    N.check(L.qex_td_make_rdm1(batch, n, _lib.p(C), _lib.p(occ), _lib.p(D), _lib.stream()),
            "qex_td_make_rdm1")
    return D[0] if single else D


def make_rdm1_masked(mo_coeff, mo_occ, mask):
    """``qedft/train/td/scf_functions_masked.py:523-543``."""
    torch = N.require_cuda()
    mask = _dev(mask, torch.bool)
    C = torch.where(mask[:, None], _dev(mo_coeff, torch.float64), 0.0)
    occ = torch.where(mask, _dev(mo_occ, torch.float64), 0.0)
    D = make_rdm1(C, occ)
    return torch.where(mask[:, None] & mask[None, :], D, 0.0)


def coulomb(factors, dm):
    torch = N.require_cuda()
    L = _lib.lib()
    naux, n, _ = factors.shape
    J = torch.empty((n, n), dtype=torch.float64, device="cuda")
    ws = torch.empty(naux * 8, dtype=torch.uint8, device="cuda")
    N.check(L.qex_td_coulomb(n, naux, _lib.p(factors), _lib.p(dm), _lib.p(J), _lib.p(ws),
                             ws.numel(), _lib.stream()), "qex_td_coulomb")
    return J


class DIIS:
    """Device-resident CDIIS history (``qedft/train/td/jax_diis.py``)."""

    def __init__(self, n, max_vec=8, min_vecs=2):
        torch = N.require_cuda()
        self.n, self.max_vec, self.min_vecs = n, max_vec, min_vecs
        self.errs = torch.empty((max_vec, n * n), dtype=torch.float64, device="cuda")
        self.focks = torch.empty((max_vec, n * n), dtype=torch.float64, device="cuda")
        self.count = 0
        self.ws = torch.empty(2 * n * n * 8, dtype=torch.uint8, device="cuda")

    def update(self, fock, dm, ovlp):
        torch = N.require_cuda()
        L = _lib.lib()
        n = self.n
        if self.count == self.max_vec:  # drop the oldest pair
            self.errs = torch.roll(self.errs, -1, 0)
            self.focks = torch.roll(self.focks, -1, 0)
            self.count -= 1
        slot = self.count
        N.check(L.qex_td_diis_error(n, _lib.p(fock), _lib.p(dm), _lib.p(ovlp),
                                    _lib.p(self.errs[slot]), _lib.p(self.ws), self.ws.numel(),
                                    _lib.stream()), "qex_td_diis_error")
        self.focks[slot].copy_(fock.reshape(-1))
        self.count += 1
        out = torch.empty((n, n), dtype=torch.float64, device="cuda")
        N.check(L.qex_td_diis_extrapolate(n, self.count, self.min_vecs, _lib.p(self.errs),
                                          _lib.p(self.focks), _lib.p(out), None, _lib.stream()),
                "qex_td_diis_extrapolate")
        return out


@dataclasses.dataclass
class ScfResult:
    energies: object  # (max_cycle,) device tensor
    dm: object
    mo_energy: object
    mo_coeff: object
    status: object
    entropic_energy: object = None  # (max_cycle,) with Fermi occupations
    mo_occ: object = None


def energy_tot(dm, h1e, J, excsum, energy_nuc):
    return (dm * h1e.T).sum() + 0.5 * (dm * J).sum() + excsum + energy_nuc


def _fermi_occ(nelectron, mo_energy, fermi):
    from .fermi import _run

    occ, entr, _, _, _ = _run(mo_energy, float(nelectron), fermi.get("theta", 0.04),
                              fermi.get("mu"), fermi.get("mu_shift", 0.001),
                              fermi.get("step_grad", 0.6), fermi.get("max_steps", 100),
                              {"optimize": 0, "jax": 1, "stable": 2}[fermi.get("mode", "stable")])
    return occ, entr


def run_scf(mol, max_cycle=30, diis_max_vec=8, diis_start_cycle=1, diis_min_vecs=2, xc="LDA",
            fermi=None):
    """Fixed-cycle SCF for one synthetic molecule (factored Coulomb; the LDA
    exchange, or a ``numint.NeuralXC`` functional as ``xc``).

    ``fermi``: None for aufbau occupations, or a dict (``theta``, ``mode`` in
    "stable" (the default: Newton from the HOMO/LUMO midpoint) / "jax" /
    "optimize" (both start just above the lowest orbital and stall when the
    gaps are many theta wide), ``max_steps``, ``step_grad``, ``mu_shift``,
    ``mu``) for Fermi-Dirac occupations in every cycle (``qedft/train/td/fermi.py``,
    the ``frac_*`` options of ``qedft/config/default_config_td.yaml``); the
    density matrix then spans all orbitals and the cycle's entropic energy
    theta sum 2[f ln f + (1-f) ln(1-f)] is returned beside the energy."""
    from .numint import GGA_CODES, eval_ao_deriv1

    torch = N.require_cuda()
    gga = isinstance(xc, str) and xc.upper().replace(" ", "") in GGA_CODES
    ao = eval_ao_deriv1(mol) if gga else _dev(mol.ao, torch.float64)
    w = _dev(mol.weights, torch.float64)
    s1e = _dev(mol.s1e, torch.float64)
    h1e = _dev(mol.h1e, torch.float64)
    fac = _dev(mol.eri_factors, torch.float64)
    n = s1e.shape[0]
    e0, c0 = generalized_eigh(h1e, s1e)

    def occupations(mo_e):
        if fermi is None:
            return get_occ(mol.nelectron, mo_e), None
        return _fermi_occ(mol.nelectron, mo_e, fermi)

    occ, _ = occupations(e0)
    dm = make_rdm1(c0, occ)

    def veff(dm):
        J = coulomb(fac, dm)
        _, excsum, vmat = nr_rks(ao, w, dm, xc)
        return J + vmat, J, excsum

    vhf, J, exc = veff(dm)
    diis = DIIS(n, diis_max_vec, diis_min_vecs)
    energies = torch.empty(max_cycle, dtype=torch.float64, device="cuda")
    status = torch.zeros(max_cycle, dtype=torch.int32, device="cuda")
    entropic = torch.zeros(max_cycle, dtype=torch.float64, device="cuda") if fermi else None
    mo_e = mo_c = None
    for cycle in range(max_cycle):
        fock = h1e + vhf
        if cycle >= diis_start_cycle:
            fock = diis.update(fock, dm, s1e)
        mo_e, mo_c, st = generalized_eigh(fock, s1e, return_status=True)
        status[cycle] = st
        occ, entr = occupations(mo_e)
        if entr is not None:
            entropic[cycle] = entr
        dm = make_rdm1(mo_c, occ)
        vhf, J, exc = veff(dm)
        energies[cycle] = energy_tot(dm, h1e, J, exc, mol.energy_nuc)
    return ScfResult(energies, dm, mo_e, mo_c, status, entropic, occ)
