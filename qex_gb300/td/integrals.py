"""Gaussian integrals and density fitting on the GPU (``ints.cu``).

Overlap, kinetic and nuclear-attraction matrices, the three-centre
(ij|P) and two-centre (P|Q) Coulomb integrals over an auxiliary basis, and the
fitted factors B_P = sum_Q (L^-1)_PQ (Q|ij) with (P|Q) = L L^T, so that
(ij|kl) ~ sum_P B_Pij B_Pkl: what pyscf's libcint and pyscfad's density
fitting give the reference (``qedft/train/td/hf.py:425-449``).  The J build of
the SCF then runs on these factors unchanged.  Cartesian s, p and d shells.
"""

from __future__ import annotations

import math

import numpy as np

from .. import _native as N
from . import _lib
from .numint import _dev


def shell_arrays(shells):
    """(centers, l, prim_offset, ao_offset, exponents, coefficients) of a shell list."""
    from .workloads import shell_arrays as arrays

    return arrays(shells)


def _nao(shells):
    from .workloads import ncart

    return sum(ncart(s.l) for s in shells)


def _prim_norm(alpha, l):
    return (2.0 * alpha / math.pi) ** 0.75 * (4.0 * alpha) ** (0.5 * l)


# even-tempered auxiliary exponents (s, p, d) per element row: a fitting set
# for the Coulomb term (the Weigend/def2 JK-fit sets pyscf uses are not in this
# image); the d set is added where the orbital basis carries d shells
AUX_S = {1: (0.15, 0.45, 1.35, 4.05), 2: (0.15, 0.45, 1.35, 4.05, 12.15, 36.45)}
AUX_P = {1: (0.4, 1.2), 2: (0.3, 0.9, 2.7)}
AUX_D = {1: (), 2: (0.5, 1.5, 4.5)}


def even_tempered_aux(mol):
    """Uncontracted normalised s and p (and, for an orbital basis with d
    shells, d) auxiliary shells on every atom."""
    from .workloads import Shell

    with_d = any(s.l == 2 for s in mol.shells)
    out = []
    for z, R in zip(mol.charges, mol.positions):
        row = 1 if int(z) <= 2 else 2
        sets = [(0, AUX_S[row]), (1, AUX_P[row])] + ([(2, AUX_D[row])] if with_d else [])
        for l, exps in sets:
            for a in exps:
                out.append(Shell(center=np.asarray(R, np.float64).copy(), l=l,
                                 exponents=np.array([a]), coefficients=np.array([_prim_norm(a, l)])))
    return out


def _args(shells):
    return [_dev(x) for x in shell_arrays(shells)]


def int1e(mol):
    """(S, T, V) device matrices: overlap, kinetic, nuclear attraction."""
    torch = N.require_cuda()
    n = mol.nao
    S, T, V = (torch.empty((n, n), dtype=torch.float64, device="cuda") for _ in range(3))
    a = _args(mol.shells)
    Z = _dev(np.asarray(mol.charges, np.float64))
    R = _dev(np.ascontiguousarray(mol.positions, np.float64).reshape(-1))
    N.check(_lib.lib().qex_td_int1e(len(mol.shells), *[_lib.p(x) for x in a], n,
                                    len(mol.charges), _lib.p(Z), _lib.p(R), _lib.p(S), _lib.p(T),
                                    _lib.p(V), _lib.stream()), "qex_td_int1e")
    return S, T, V


def int3c2e(mol, aux):
    """(naux, n, n) device tensor (ij|P)."""
    torch = N.require_cuda()
    n, na = mol.nao, _nao(aux)
    out = torch.empty((na, n, n), dtype=torch.float64, device="cuda")
    a, b = _args(mol.shells), _args(aux)
    N.check(_lib.lib().qex_td_int3c2e(len(mol.shells), *[_lib.p(x) for x in a], n, len(aux),
                                      *[_lib.p(x) for x in b], na, _lib.p(out), _lib.stream()),
            "qex_td_int3c2e")
    return out


def int2c2e(aux):
    """(naux, naux) device tensor (P|Q)."""
    torch = N.require_cuda()
    na = _nao(aux)
    out = torch.empty((na, na), dtype=torch.float64, device="cuda")
    b = _args(aux)
    N.check(_lib.lib().qex_td_int2c2e(len(aux), *[_lib.p(x) for x in b], na, _lib.p(out),
                                      _lib.stream()), "qex_td_int2c2e")
    return out


def df_factors(mol, aux=None):
    """B (naux, n, n) with (ij|kl) ~ sum_P B_Pij B_Pkl: Cholesky of (P|Q) and a
    forward substitution of (Q|ij), both on the GPU."""
    torch = N.require_cuda()
    aux = even_tempered_aux(mol) if aux is None else aux
    B = int3c2e(mol, aux)
    V = int2c2e(aux)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    na, n = B.shape[0], B.shape[1]
    N.check(_lib.lib().qex_td_df_factors(na, n * n, _lib.p(V), _lib.p(B), _lib.p(st),
                                         _lib.stream()), "qex_td_df_factors")
    if int(st.item()) != 0:
        raise ValueError("the auxiliary metric (P|Q) is not positive definite")
    return B
