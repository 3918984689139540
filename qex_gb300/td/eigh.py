"""Generalized symmetric eigensolver on the GPU.

``generalized_eigh`` mirrors ``qedft/train/td/generalized_eigensolver.py:264-330``
(symmetrise, SPD shift of S when its smallest eigenvalue is below 1e-12,
Cholesky, C = L^-1 A L^-T, eigh(C), V = L^-T U); ``masked_generalized_eigh``
mirrors ``qedft/train/td/generalized_eigensolver_masked.py:19-89`` (padded
diagonals 1e-12, padded slots sorted last and zeroed).  Batched: A and S may
be (batch, n, n).
"""

from __future__ import annotations

from .. import _native as N
from . import _lib
from .numint import _dev


def generalized_eigh(A, B, *, eps: float = 1.0e-12, return_status: bool = False):
    torch = N.require_cuda()
    if eps != 1.0e-12:
        raise NotImplementedError("the GPU solver uses the reference's eps = 1e-12")
    L = _lib.lib()
    A = _dev(A, torch.float64)
    B = _dev(B, torch.float64)
    single = A.dim() == 2
    if single:
        A, B = A[None], B[None]
    batch, n, _ = A.shape
    w = torch.empty((batch, n), dtype=torch.float64, device="cuda")
    V = torch.empty((batch, n, n), dtype=torch.float64, device="cuda")
    st = torch.empty(batch, dtype=torch.int32, device="cuda")  # every entry written by the solver
    ws = torch.empty(L.qex_td_gen_eigh_workspace_size(batch, n), dtype=torch.uint8, device="cuda")
    N.check(L.qex_td_gen_eigh(batch, n, _lib.p(A), _lib.p(B), _lib.p(w), _lib.p(V), _lib.p(st),
                              _lib.p(ws), ws.numel(), _lib.stream()), "qex_td_gen_eigh")
    if single:
        w, V, st = w[0], V[0], st[0]
    return (w, V, st) if return_status else (w, V)


_PATHS = {}  # n -> (selected path, {path: ms})


def set_path(n: int, path: int) -> None:
    """Select the mixed-precision solver's path for matrices of size n: 0 the
    default, 1 the shared-memory FP32 solve (n <= 128), 2 the FP64 factor and
    tridiagonal stage (``qex_td_gen_eigh_set_path``)."""
    N.check(_lib.lib().qex_td_gen_eigh_set_path(int(n), int(path)), "qex_td_gen_eigh_set_path")


def tune_path(A, B, repeats: int = 3):
    """Autotune the eigensolver path for the size of (A, B): time each
    candidate path on this pair (CUDA events, median of ``repeats`` after one
    warm-up) and keep the faster for that size.  Both paths refine to the same
    FP64 accuracy.  Cached per size; returns (path, {path: ms})."""
    torch = N.require_cuda()
    A = _dev(A, torch.float64)
    n = A.shape[-1]
    if n in _PATHS:
        return _PATHS[n]
    if n > 240:
        _PATHS[n] = (0, {})
        return _PATHS[n]
    cands = (1, 2) if n <= 128 else (2,)
    timings = {}
    stream = torch.cuda.current_stream()
    for path in cands:
        set_path(n, path)
        generalized_eigh(A, B)
        ts = []
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            generalized_eigh(A, B)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        timings[path] = sorted(ts)[len(ts) // 2]
    best = min(timings, key=timings.get)
    set_path(n, best)
    _PATHS[n] = (best, timings)
    return _PATHS[n]


def masked_generalized_eigh(fock, s1e, mask):
    """Padded/masked solve with the reference's padding and sorting rules
    (``qex_td_mask_pad``, the solve, ``qex_td_mask_sort``)."""
    torch = N.require_cuda()
    L = _lib.lib()
    fock = _dev(fock, torch.float64).contiguous()
    s1e = _dev(s1e, torch.float64).contiguous()
    mask8 = _dev(mask, torch.bool).to(torch.uint8).contiguous()
    n = fock.shape[-1]
    f = torch.empty_like(fock)
    s = torch.empty_like(s1e)
    N.check(L.qex_td_mask_pad(n, _lib.p(fock), _lib.p(s1e), _lib.p(mask8), _lib.p(f), _lib.p(s),
                              _lib.stream()), "qex_td_mask_pad")
    w, v = generalized_eigh(f, s)
    w_out = torch.empty_like(w)
    v_out = torch.empty_like(v)
    N.check(L.qex_td_mask_sort(n, _lib.p(w), _lib.p(v.contiguous()), _lib.p(mask8), _lib.p(w_out),
                               _lib.p(v_out), _lib.stream()), "qex_td_mask_sort")
    return w_out, v_out
