"""ctypes signatures of ``include/qex_td.h``."""

from __future__ import annotations

import ctypes

from .. import _native as N

_v = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_sz = ctypes.c_size_t

SIGNATURES = {
    "qex_td_eval_ao": (ctypes.c_int, [_i64, _v, _i32, _v, _v, _v, _v, _v, _v, _i32, _v, _v]),
    "qex_td_rho_workspace_size": (_sz, [_i64, _i32]),
    "qex_td_rho": (ctypes.c_int, [_i64, _i32, _v, _v, _v, _v, _sz, _v]),
    "qex_td_lda_workspace_size": (_sz, [_i64]),
    "qex_td_lda": (ctypes.c_int, [_i64, _v, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_lda_vwn": (ctypes.c_int, [_i64, _v, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_vxc_workspace_size": (_sz, [_i64, _i32]),
    "qex_td_vxc": (ctypes.c_int, [_i64, _i32, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_gen_eigh_workspace_size": (_sz, [_i32, _i32]),
    "qex_td_gen_eigh": (ctypes.c_int, [_i32, _i32, _v, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_make_rdm1": (ctypes.c_int, [_i32, _i32, _v, _v, _v, _v]),
    "qex_td_eval_ao_deriv1": (ctypes.c_int, [_i64, _v, _i32, _v, _v, _v, _v, _v, _v, _i32, _v,
                                             _v]),
    "qex_td_rho_gga_workspace_size": (_sz, [_i64, _i32]),
    "qex_td_rho_gga": (ctypes.c_int, [_i64, _i32, _v, _v, _v, _v, _sz, _v]),
    "qex_td_gga_pbe_x_workspace_size": (_sz, [_i64]),
    "qex_td_gga_pbe_x": (ctypes.c_int, [_i64, _v, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_vxc_gga_workspace_size": (_sz, [_i64, _i32]),
    "qex_td_vxc_gga": (ctypes.c_int, [_i64, _i32, _v, _v, _v, _v, _sz, _v]),
    "qex_td_becke_grid": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _v, _v, _i32, _v, _v, _i32,
                                         _i64, _v, _v, _v]),
    "qex_td_int1e": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _v, _i32, _i32, _v, _v, _v, _v,
                                    _v, _v]),
    "qex_td_int3c2e": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _v, _i32, _i32, _v, _v, _v, _v,
                                      _v, _v, _i32, _v, _v]),
    "qex_td_int2c2e": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _v, _i32, _v, _v]),
    "qex_td_df_factors": (ctypes.c_int, [_i32, _i64, _v, _v, _v, _v]),
    "qex_td_fermi_occupations": (ctypes.c_int, [_i32, _i32, _v, _v, ctypes.c_double, _v,
                                                ctypes.c_double, ctypes.c_double, _i32, _i32,
                                                _v, _v, _v, _v, _v, _v]),
    "qex_td_diis_error": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_diis_extrapolate": (ctypes.c_int, [_i32, _i32, _i32, _v, _v, _v, _v, _v]),
    "qex_td_coulomb": (ctypes.c_int, [_i32, _i32, _v, _v, _v, _v, _sz, _v]),
    "qex_td_nn_xc_workspace_size": (_sz, [_i64, _i32]),
    "qex_td_nn_xc_global_workspace_size": (_sz, [_i64, _i32]),
    "qex_td_nn_xc_global": (ctypes.c_int, [_i64, _i32, _v, _v, _v, ctypes.c_double, _v, _v, _v,
                                           _sz, _v]),
    "qex_td_nn_xc": (ctypes.c_int, [_i64, _i32, _v, _v, _v, ctypes.c_double, _v, _v, _v, _v,
                                    _sz, _v]),
    "qex_td_fock_energy": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, ctypes.c_double, _v, _v, _v]),
    "qex_td_orbital_gradient_workspace_size": (_sz, [_i32]),
    "qex_td_orbital_gradient": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _sz, _v]),
    "qex_td_scf_check": (ctypes.c_int, [_i32, _i32, _v, _v, _v, ctypes.c_double, ctypes.c_double,
                                        _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v]),
    "qex_td_aufbau_occ": (ctypes.c_int, [_i32, _i32, _v, _i32, _v, _v]),
    "qex_td_mask_pad": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _v]),
    "qex_td_mask_sort": (ctypes.c_int, [_i32, _v, _v, _v, _v, _v, _v]),
    "qex_td_gen_eigh_set_path": (ctypes.c_int, [_i32, _i32]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = N.load()
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def stream():
    torch = N.require_cuda()
    return torch.cuda.current_stream().cuda_stream


def p(t):
    return None if t is None else t.data_ptr()
