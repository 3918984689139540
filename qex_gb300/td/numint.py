"""Numerical integration pieces of the 3D Kohn-Sham path on the GPU.

Mirrors ``qedft/train/td/numint_legacy.py``: ``eval_ao`` (AO values),
``eval_rho`` (:351-397), ``nr_rks`` (:122-348, LDA branch :148-164 with the
``vmat + vmat^T`` symmetrisation of :337).  Arrays are torch CUDA tensors
(float64, row-major); every call runs the kernels of ``include/qex_td.h``.
"""

from __future__ import annotations

import numpy as np

from .. import _native as N
from . import _lib


def _dev(a, dtype=None):
    torch = N.require_cuda()
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=dtype or a.dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda", dtype=dtype)


def eval_ao(mol, coords=None):
    """(G, nao) AO values of ``mol``'s Cartesian contracted shells on ``coords``."""
    torch = N.require_cuda()
    L = _lib.lib()
    coords = _dev(mol.coords if coords is None else coords, torch.float64)
    centers, l, poff, aoff, ex, co = mol.shell_arrays()
    G = coords.shape[0]
    ao = torch.empty((G, mol.nao), dtype=torch.float64, device="cuda")
    args = [_dev(x) for x in (centers, l, poff, aoff, ex, co)]
    rc = L.qex_td_eval_ao(G, _lib.p(coords), len(mol.shells), *[_lib.p(a) for a in args],
                          mol.nao, _lib.p(ao), _lib.stream())
    N.check(rc, "qex_td_eval_ao")
    return ao


def eval_rho(ao, dm):
    """rho_g = sum_ij ao_gi D_ij ao_gj (LDA)."""
    torch = N.require_cuda()
    L = _lib.lib()
    ao = _dev(ao, torch.float64)
    dm = _dev(dm, torch.float64)
    G, n = ao.shape
    ws = torch.empty(max(L.qex_td_rho_workspace_size(G, n), 8), dtype=torch.uint8, device="cuda")
    rho = torch.empty(G, dtype=torch.float64, device="cuda")
    N.check(L.qex_td_rho(G, n, _lib.p(ao), _lib.p(dm), _lib.p(rho), _lib.p(ws), ws.numel(),
                         _lib.stream()), "qex_td_rho")
    return rho


def eval_xc_lda(rho, weights):
    """(exc, vrho, nelec, excsum) of the Slater exchange on the grid."""
    torch = N.require_cuda()
    L = _lib.lib()
    rho = _dev(rho, torch.float64)
    weights = _dev(weights, torch.float64)
    G = rho.shape[0]
    exc = torch.empty_like(rho)
    vrho = torch.empty_like(rho)
    sums = torch.empty(2, dtype=torch.float64, device="cuda")
    ws = torch.empty(L.qex_td_lda_workspace_size(G), dtype=torch.uint8, device="cuda")
    N.check(L.qex_td_lda(G, _lib.p(rho), _lib.p(weights), _lib.p(exc), _lib.p(vrho), _lib.p(sums),
                         _lib.p(ws), ws.numel(), _lib.stream()), "qex_td_lda")
    return exc, vrho, sums[0], sums[1]


def vxc_matrix(ao, weights, vrho):
    """ao^T diag(0.5 w v) ao + its transpose."""
    torch = N.require_cuda()
    L = _lib.lib()
    ao = _dev(ao, torch.float64)
    G, n = ao.shape
    vmat = torch.empty((n, n), dtype=torch.float64, device="cuda")
    ws = torch.empty(max(L.qex_td_vxc_workspace_size(G, n), 8), dtype=torch.uint8, device="cuda")
    N.check(L.qex_td_vxc(G, n, _lib.p(ao), _lib.p(_dev(weights, torch.float64)),
                         _lib.p(_dev(vrho, torch.float64)), _lib.p(vmat), _lib.p(ws), ws.numel(),
                         _lib.stream()), "qex_td_vxc")
    return vmat


def nr_rks(ao, weights, dm, xc_code="LDA"):
    """(nelec, excsum, vmat) for the LDA exchange (``numint_legacy.py:122-164,337``)."""
    if xc_code.upper() not in ("LDA", "LDA_X", "SLATER"):
        raise NotImplementedError(f"xc_code {xc_code!r}: the GPU path implements the LDA exchange")
    rho = eval_rho(ao, dm)
    exc, vrho, nelec, excsum = eval_xc_lda(rho, weights)
    return nelec, excsum, vxc_matrix(ao, weights, vrho)
