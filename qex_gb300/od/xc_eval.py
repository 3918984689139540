"""GPU evaluation of a 1D XC functional on given densities (``include/qex_xc1d.h``)."""

from __future__ import annotations

import ctypes

import numpy as np

from .. import _native as N
from ..xc import resolve
from . import utils

_SIG = (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p, ctypes.POINTER(N.XcSpec), ctypes.c_void_p,
                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_size_t, ctypes.c_void_p])


_KSR_SIG = (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.POINTER(N.XcSpec), ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p])


def _lib():
    lib = N.load()
    fn = lib.qex_xc1d_eval
    fn.restype, fn.argtypes = _SIG
    lib.qex_xc1d_workspace_size.restype = ctypes.c_int
    lib.qex_xc1d_workspace_size.argtypes = [ctypes.c_int64, ctypes.POINTER(N.XcSpec),
                                            ctypes.POINTER(ctypes.c_size_t)]
    lib.qex_ksr1d_eval.restype, lib.qex_ksr1d_eval.argtypes = _KSR_SIG
    return lib


def ksr_eval(densities, grid_spacing, xc_energy_density_fn, convention="local", potential=True):
    """Batched KSR evaluation on the GPU: ``densities`` is a list of 1D arrays
    (any lengths, each molecule on its own grid spacing).  Returns per-molecule
    (E_xc, v_xc or None, eps) as host arrays.  The network runs on
    ``qex_ksr1d_eval`` (one warp per molecule)."""
    torch = N.require_cuda()
    lib = _lib()
    functional, params = resolve(xc_energy_density_fn)
    if functional.kind != N.QEX_XC_KSR:
        raise TypeError("ksr_eval needs a KSR functional")
    conv = {"amplitude": N.QEX_XC_AMPLITUDE, "local": N.QEX_XC_LOCAL}[convention]
    spec, keep = functional.spec(params, conv)
    dens = [np.ascontiguousarray(d, dtype=np.float64).reshape(-1) for d in densities]
    sizes = np.array([d.size for d in dens], dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum(sizes[:-1])]).astype(np.int64)
    dev = torch.device("cuda")
    d = torch.as_tensor(np.concatenate(dens), device=dev)
    ng = torch.as_tensor(sizes, device=dev)
    off = torch.as_tensor(offs, device=dev)
    dx = torch.as_tensor(np.broadcast_to(np.asarray(grid_spacing, np.float64), sizes.shape).copy(),
                         device=dev)
    vals = torch.empty_like(d)
    pot = torch.empty_like(d) if potential else None
    energy = torch.empty(len(dens), dtype=torch.float64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.qex_ksr1d_eval(len(dens), int(sizes.max()), ng.data_ptr(), off.data_ptr(),
                            dx.data_ptr(), ctypes.byref(spec), d.data_ptr(), vals.data_ptr(),
                            pot.data_ptr() if pot is not None else None, energy.data_ptr(), stream)
    N.check(rc, "qex_ksr1d_eval")
    torch.cuda.current_stream().synchronize()
    del keep
    e = energy.cpu().numpy()
    v = pot.cpu().numpy() if pot is not None else None
    f = vals.cpu().numpy()
    out = []
    for i, (o, n) in enumerate(zip(offs, sizes)):
        out.append((float(e[i]), None if v is None else v[o:o + n], f[o:o + n]))
    return out


def xc_energy_and_potential(density, xc_energy_density_fn, grids, convention="amplitude"):
    """(E_xc, v_xc, f) for one density on ``grids`` (host arrays in and out)."""
    torch = N.require_cuda()
    lib = _lib()
    functional, params = resolve(xc_energy_density_fn)
    if functional.kind == N.QEX_XC_KSR:
        return ksr_eval([density], utils.get_dx(grids), xc_energy_density_fn, convention)[0]
    conv = {"amplitude": N.QEX_XC_AMPLITUDE, "local": N.QEX_XC_LOCAL}[convention]
    spec, keep = functional.spec(params, conv)
    n = np.ascontiguousarray(density, dtype=np.float64).reshape(-1)
    dev = torch.device("cuda")
    d = torch.as_tensor(n, device=dev)
    ng = torch.tensor([n.size], dtype=torch.int32, device=dev)
    off = torch.zeros(1, dtype=torch.int64, device=dev)
    dx = torch.tensor([utils.get_dx(grids)], dtype=torch.float64, device=dev)
    vals = torch.empty_like(d)
    pot = torch.empty_like(d)
    energy = torch.empty(1, dtype=torch.float64, device=dev)
    need = ctypes.c_size_t()
    N.check(lib.qex_xc1d_workspace_size(n.size, ctypes.byref(spec), ctypes.byref(need)),
            "qex_xc1d_workspace_size")
    ws = torch.empty(max(need.value, 16), dtype=torch.uint8, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.qex_xc1d_eval(1, n.size, ng.data_ptr(), off.data_ptr(), dx.data_ptr(),
                           ctypes.byref(spec), d.data_ptr(), vals.data_ptr(), pot.data_ptr(),
                           energy.data_ptr(), ws.data_ptr(), ws.numel(), stream)
    N.check(rc, "qex_xc1d_eval")
    torch.cuda.current_stream().synchronize()
    del keep
    return float(energy.cpu()[0]), pot.cpu().numpy(), vals.cpu().numpy()
