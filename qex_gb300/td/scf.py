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


def get_occ(nelectron, mo_energy, out=None):
    """2 electrons in each of the lowest Ne/2 orbitals (ties by index), one
    kernel (``qex_td_aufbau_occ``); mo_energy may be (batch, n)."""
    torch = N.require_cuda()
    mo_energy = _dev(mo_energy, torch.float64).contiguous()
    n = mo_energy.shape[-1]
    batch = mo_energy.numel() // n
    occ = torch.empty_like(mo_energy) if out is None else out
    N.check(_lib.lib().qex_td_aufbau_occ(batch, n, _lib.p(mo_energy), int(nelectron),
                                         _lib.p(occ), _lib.stream()), "qex_td_aufbau_occ")
    return occ


def orbital_gradient_norm(mo_coeff, mo_occ, fock):
    """|g| with g = 2 C_vir^T F C_occ (pyscf's RHF ``get_grad``, as the
    reference's loop calls it at ``qedft/train/td/hf.py:81-84``), as a (1,)
    device tensor."""
    torch = N.require_cuda()
    L = _lib.lib()
    C = _dev(mo_coeff, torch.float64).contiguous()
    occ = _dev(mo_occ, torch.float64).contiguous()
    F = _dev(fock, torch.float64).contiguous()
    n = C.shape[0]
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    ws = torch.empty(L.qex_td_orbital_gradient_workspace_size(n), dtype=torch.uint8, device="cuda")
    N.check(L.qex_td_orbital_gradient(n, _lib.p(C), _lib.p(occ), _lib.p(F), _lib.p(out),
                                      _lib.p(ws), ws.numel(), _lib.stream()),
            "qex_td_orbital_gradient")
    return out


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
    """Device-resident CDIIS history (``qedft/train/td/jax_diis.py``) in a
    ring of ``max_vec`` slots: the newest pair overwrites the oldest once the
    ring is full, and the extrapolation (whose result does not depend on the
    order of the pairs) reads the filled slots in place."""

    def __init__(self, n, max_vec=8, min_vecs=2):
        torch = N.require_cuda()
        self.n, self.max_vec, self.min_vecs = n, max_vec, min_vecs
        self.errs = torch.empty((max_vec, n * n), dtype=torch.float64, device="cuda")
        self.focks = torch.empty((max_vec, n * n), dtype=torch.float64, device="cuda")
        self.total = 0
        self.ws = torch.empty(2 * n * n * 8, dtype=torch.uint8, device="cuda")

    @property
    def count(self):
        return min(self.total, self.max_vec)

    def update(self, fock, dm, ovlp):
        torch = N.require_cuda()
        L = _lib.lib()
        n = self.n
        slot = self.total % self.max_vec
        N.check(L.qex_td_diis_error(n, _lib.p(fock), _lib.p(dm), _lib.p(ovlp),
                                    _lib.p(self.errs[slot]), _lib.p(self.ws), self.ws.numel(),
                                    _lib.stream()), "qex_td_diis_error")
        self.focks[slot].copy_(fock.reshape(-1))
        self.total += 1
        out = torch.empty((n, n), dtype=torch.float64, device="cuda")
        N.check(L.qex_td_diis_extrapolate(n, self.count, self.min_vecs, _lib.p(self.errs),
                                          _lib.p(self.focks), _lib.p(out), None, _lib.stream()),
                "qex_td_diis_extrapolate")
        return out


@dataclasses.dataclass
class ScfResult:
    energies: object  # (max_cycle,) device tensor, every cycle run
    dm: object        # dm, mo_energy, mo_coeff, mo_occ, e_tot: the first converged
    mo_energy: object  # cycle's (where the reference's loop stops), else the last
    mo_coeff: object
    status: object
    entropic_energy: object = None  # (max_cycle,) with Fermi occupations
    mo_occ: object = None
    e_tot: object = None       # (1,) device tensor
    converged: object = None   # device int32 state: [converged, first converged cycle, cycles]
    grad_norms: object = None  # (max_cycle,) |g| of every cycle


def energy_tot(dm, h1e, J, excsum, energy_nuc):
    """E = tr(D h^T) + 1/2 tr(D J) + E_xc + E_nuc on the device (one kernel)."""
    torch = N.require_cuda()
    n = dm.shape[-1]
    zero = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    e = torch.empty(1, dtype=torch.float64, device="cuda")
    exc = _dev(excsum, torch.float64).reshape(1).contiguous()
    N.check(_lib.lib().qex_td_fock_energy(n, _lib.p(h1e), _lib.p(J), _lib.p(zero), _lib.p(dm),
                                          _lib.p(exc), float(energy_nuc), None, _lib.p(e),
                                          _lib.stream()), "qex_td_fock_energy")
    return e[0]


def _fermi_occ(nelectron, mo_energy, fermi):
    from .fermi import _run

    occ, entr, _, _, _ = _run(mo_energy, float(nelectron), fermi.get("theta", 0.04),
                              fermi.get("mu"), fermi.get("mu_shift", 0.001),
                              fermi.get("step_grad", 0.6), fermi.get("max_steps", 100),
                              {"optimize": 0, "jax": 1, "stable": 2}[fermi.get("mode", "stable")])
    return occ, entr


def run_scf(mol, max_cycle=30, diis_max_vec=8, diis_start_cycle=1, diis_min_vecs=2, xc="LDA",
            fermi=None, conv_tol=1e-10, conv_tol_grad=None, early_exit=False):
    """SCF for one synthetic molecule (factored Coulomb; the LDA exchange, or a
    ``numint.NeuralXC`` functional as ``xc``), following the cycle of
    ``qedft/train/td/hf.py:47-110``: fock (DIIS from ``diis_start_cycle``),
    eigensolve, occupations, density matrix, veff, energy, then the stop rule
    |E - E_last| < ``conv_tol`` and |g| < ``conv_tol_grad`` (default
    sqrt(conv_tol)) with the orbital gradient of the new Fock matrix.

    Every step is a kernel and nothing waits on the host, so the loop can be
    captured as a CUDA graph: it runs ``max_cycle`` cycles and the results
    (``dm``, ``mo_*``, ``e_tot``) are latched at the first converged cycle,
    which is where the reference's loop stops; ``early_exit`` instead reads the
    flag on the host after every cycle and stops there (not under capture).

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
    L = _lib.lib()
    if conv_tol_grad is None:
        conv_tol_grad = float(np.sqrt(conv_tol))
    gga = isinstance(xc, str) and xc.upper().replace(" ", "") in GGA_CODES
    ao = eval_ao_deriv1(mol) if gga else _dev(mol.ao, torch.float64)
    w = _dev(mol.weights, torch.float64)
    s1e = _dev(mol.s1e, torch.float64)
    h1e = _dev(mol.h1e, torch.float64)
    fac = _dev(mol.eri_factors, torch.float64)
    n = s1e.shape[0]
    f64 = dict(dtype=torch.float64, device="cuda")
    e0, c0 = generalized_eigh(h1e, s1e)

    def occupations(mo_e):
        if fermi is None:
            return get_occ(mol.nelectron, mo_e), None
        return _fermi_occ(mol.nelectron, mo_e, fermi)

    fock = torch.empty((n, n), **f64)

    def veff_fock_energy(dm, energy_out):
        """The new Fock matrix h1e + J + Vxc and the energy of dm (one kernel)."""
        J = coulomb(fac, dm)
        _, excsum, vmat = nr_rks(ao, w, dm, xc)
        exc = excsum.reshape(1) if hasattr(excsum, "reshape") else torch.tensor([excsum], **f64)
        N.check(L.qex_td_fock_energy(n, _lib.p(h1e), _lib.p(J), _lib.p(vmat), _lib.p(dm),
                                     _lib.p(exc), float(mol.energy_nuc), _lib.p(fock),
                                     _lib.p(energy_out), _lib.stream()), "qex_td_fock_energy")

    occ, _ = occupations(e0)
    dm = make_rdm1(c0, occ)
    e_init = torch.empty(1, **f64)
    veff_fock_energy(dm, e_init)
    diis = DIIS(n, diis_max_vec, diis_min_vecs)
    energies = torch.empty(max_cycle, **f64)
    gnorms = torch.empty(max_cycle, **f64)
    status = torch.zeros(max_cycle, dtype=torch.int32, device="cuda")
    state = torch.zeros(3, dtype=torch.int32, device="cuda")
    entropic = torch.zeros(max_cycle, **f64) if fermi else None
    dm_out, mo_c_out = torch.empty((n, n), **f64), torch.empty((n, n), **f64)
    mo_e_out, occ_out, e_tot = torch.empty(n, **f64), torch.empty(n, **f64), torch.empty(1, **f64)
    gws = torch.empty(L.qex_td_orbital_gradient_workspace_size(n), dtype=torch.uint8, device="cuda")
    for cycle in range(max_cycle):
        f_in = diis.update(fock, dm, s1e) if cycle >= diis_start_cycle else fock.clone()
        mo_e, mo_c, st = generalized_eigh(f_in, s1e, return_status=True)
        status[cycle] = st
        occ, entr = occupations(mo_e)
        if entr is not None:
            entropic[cycle] = entr
        dm = make_rdm1(mo_c, occ)
        veff_fock_energy(dm, energies[cycle:cycle + 1])
        N.check(L.qex_td_orbital_gradient(n, _lib.p(mo_c), _lib.p(occ), _lib.p(fock),
                                          _lib.p(gnorms[cycle:cycle + 1]), _lib.p(gws),
                                          gws.numel(), _lib.stream()), "qex_td_orbital_gradient")
        N.check(L.qex_td_scf_check(cycle, n, _lib.p(energies), _lib.p(e_init),
                                   _lib.p(gnorms[cycle:cycle + 1]), float(conv_tol),
                                   float(conv_tol_grad), _lib.p(state), _lib.p(dm),
                                   _lib.p(mo_e), _lib.p(mo_c), _lib.p(occ), _lib.p(dm_out),
                                   _lib.p(mo_e_out), _lib.p(mo_c_out), _lib.p(occ_out),
                                   _lib.p(e_tot), _lib.stream()), "qex_td_scf_check")
        if early_exit and int(state[0].item()):
            energies = energies[:cycle + 1]
            gnorms = gnorms[:cycle + 1]
            status = status[:cycle + 1]
            if entropic is not None:
                entropic = entropic[:cycle + 1]
            break
    return ScfResult(energies, dm_out, mo_e_out, mo_c_out, status, entropic, occ_out, e_tot, state,
                     gnorms)
