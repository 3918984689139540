"""ctypes binding of the C ABI in ``include/qex_ks1d.h`` (and friends).

The shared library is the only compute path: if it cannot be loaded, or no
CUDA device is present, every entry point raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import threading

from . import build as _build

QEX_OK = 0
QEX_BAD_ARG = 1
QEX_NOT_CONVERGED = 2
QEX_NUMERICAL = 3
QEX_OOM = 4
QEX_TIMEOUT = 5
QEX_CUDA_ERROR = 6
QEX_FLAG_DEGENERATE_FRONTIER = 0x100
QEX_FLAG_REFINE_CAP = 0x200

QEX_INTERACTION_EXPONENTIAL = 0
QEX_INTERACTION_SOFT_COULOMB = 1
QEX_XC_NONE = 0
QEX_XC_LDA_EXP_COULOMB = 1
QEX_XC_POWER = 2
QEX_XC_WINDOW_MLP = 3
QEX_XC_KSR = 4
QEX_XC_LOCAL_MLP = 5
QEX_XC_GLOBAL_MLP = 6
QEX_NN_ACTIVATIONS = {"tanh": 0, "relu": 1, "softplus": 2, "sigmoid": 3, "elu": 4,
                      "leaky_relu": 5, "selu": 6, "gelu": 7}
QEX_NN_SELF_INTERACTION = 1
QEX_NN_NEGATIVITY = 2
QEX_NN_MAX_WIDTH = 128
QEX_XC_AMPLITUDE = 0
QEX_XC_LOCAL = 1

MAX_EIGENPAIRS = 16
MLP_WINDOW = 17
MLP_HIDDEN = 16
MLP_NUM_PARAMS = 17 * 16 + 16 + 16 * 16 + 16 + 16 + 1
KSR_CHANNELS = 16


def ksr_num_params(channels: int) -> int:
    return 6 * channels * channels + 2 * channels


_c_p = ctypes.c_void_p


class XcSpec(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("convention", ctypes.c_int32),
        ("coefficient", ctypes.c_double),
        ("power", ctypes.c_double),
        ("shift", ctypes.c_double),
        ("lda_amplitude", ctypes.c_double),
        ("lda_kappa", ctypes.c_double),
        ("normalization", ctypes.c_double),
        ("mlp_params_host", ctypes.POINTER(ctypes.c_float)),
        ("ksr_params", _c_p),
        ("ksr_minval", ctypes.c_double),
        ("ksr_maxval", ctypes.c_double),
        ("ksr_channels", ctypes.c_int32),
        ("nn_params", _c_p),
        ("nn_width", ctypes.c_int32),
        ("nn_layers", ctypes.c_int32),
        ("nn_activation", ctypes.c_int32),
        ("nn_inputs", ctypes.c_int32),
        ("nn_flags", ctypes.c_int32),
        ("mlp_params64", _c_p),
    ]


class Ks1dOptions(ctypes.Structure):
    _fields_ = [
        ("stencil", ctypes.c_int32),
        ("interaction", ctypes.c_int32),
        ("interaction_a", ctypes.c_double),
        ("interaction_b", ctypes.c_double),
        ("num_iterations", ctypes.c_int32),
        ("alpha", ctypes.c_double),
        ("alpha_decay", ctypes.c_double),
        ("num_mixing_iterations", ctypes.c_int32),
        ("density_mse_converge_tolerance", ctypes.c_double),
        ("convergence_rule", ctypes.c_int32),
        ("enforce_reflection_symmetry", ctypes.c_int32),
        ("external_potential_given", ctypes.c_int32),
        ("max_num_grids", ctypes.c_int32),
        ("max_num_electrons", ctypes.c_int32),
        ("max_nuclei", ctypes.c_int32),
        ("solve_planes", ctypes.c_int32),
        ("solve_chunk", ctypes.c_int32),
    ]


class Ks1dBatch(ctypes.Structure):
    _fields_ = [
        ("num_molecules", ctypes.c_int32),
        ("num_grids", _c_p),
        ("grid_offsets", _c_p),
        ("grid_start", _c_p),
        ("grid_spacing", _c_p),
        ("num_electrons", _c_p),
        ("num_nuclei", _c_p),
        ("locations", _c_p),
        ("nuclear_charges", _c_p),
        ("external_potential", _c_p),
        ("initial_density", _c_p),
        ("order", _c_p),
    ]


class Ks1dOutputs(ctypes.Structure):
    _fields_ = [
        ("total_energy", _c_p),
        ("gap", _c_p),
        ("converged", _c_p),
        ("density", _c_p),
        ("hartree_potential", _c_p),
        ("xc_potential", _c_p),
        ("xc_energy_density", _c_p),
        ("final_density", _c_p),
        ("external_potential_out", _c_p),
        ("status", _c_p),
        ("iterations_run", _c_p),
        ("stats", _c_p),
        ("phase_cycles", _c_p),
    ]


_SIGNATURES = {
    "qex_ks1d_workspace_size": (ctypes.c_int, [ctypes.POINTER(Ks1dOptions), ctypes.c_int32,
                                               ctypes.POINTER(ctypes.c_size_t)]),
    "qex_ks1d_workspace_size_xc": (ctypes.c_int, [ctypes.POINTER(Ks1dOptions),
                                                  ctypes.POINTER(XcSpec), ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_size_t)]),
    "qex_ks1d_solve": (ctypes.c_int, [ctypes.POINTER(Ks1dBatch), ctypes.POINTER(Ks1dOptions),
                                      ctypes.POINTER(XcSpec), ctypes.POINTER(Ks1dOutputs), _c_p,
                                      ctypes.c_size_t, _c_p]),
    "qex_ks1d_iteration": (ctypes.c_int, [ctypes.POINTER(Ks1dBatch), ctypes.POINTER(Ks1dOptions),
                                          ctypes.POINTER(XcSpec), _c_p,
                                          ctypes.POINTER(Ks1dOutputs), _c_p, ctypes.c_size_t,
                                          _c_p]),
    "qex_ks1d_noninteracting": (ctypes.c_int, [ctypes.POINTER(Ks1dBatch),
                                               ctypes.POINTER(Ks1dOptions), _c_p, _c_p, _c_p,
                                               _c_p, _c_p, _c_p, ctypes.c_size_t, _c_p]),
    "qex_probe_workspace_size": (ctypes.c_size_t, []),
    "qex_probe_fma_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double), _c_p, ctypes.c_size_t,
                                          _c_p]),
    "qex_probe_dmma_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double), _c_p, ctypes.c_size_t,
                                           _c_p]),
    "qex_version": (ctypes.c_char_p, []),
    "qex_last_launch_count": (ctypes.c_int, []),
}

_lock = threading.Lock()
_lib = None


def load(build_if_needed: bool = True) -> ctypes.CDLL:
    """Load (building first if sources changed) the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_needed and _build.needs_build():
            _build.build()
        path = _build.library_path()
        if not path.exists():
            raise RuntimeError(f"qex_gb300 native library missing at {path}; run qex_gb300.build.build()")
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def measure_fma_peak():
    """(FP64, FP32) FMA throughput in TFLOP/s on the current device."""
    torch = require_cuda()
    lib = load()
    ws = torch.empty(lib.qex_probe_workspace_size(), dtype=torch.uint8, device="cuda")
    f64, f32 = ctypes.c_double(), ctypes.c_double()
    check(lib.qex_probe_fma_peak(ctypes.byref(f64), ctypes.byref(f32), ws.data_ptr(), ws.numel(),
                                 torch.cuda.current_stream().cuda_stream), "qex_probe_fma_peak")
    return f64.value, f32.value


def measure_dmma_peak():
    """(m8n8k4, m16n8k16) FP64 tensor-core MMA throughput in TFLOP/s."""
    torch = require_cuda()
    lib = load()
    ws = torch.empty(lib.qex_probe_workspace_size(), dtype=torch.uint8, device="cuda")
    a, b = ctypes.c_double(), ctypes.c_double()
    check(lib.qex_probe_dmma_peak(ctypes.byref(a), ctypes.byref(b), ws.data_ptr(), ws.numel(),
                                  torch.cuda.current_stream().cuda_stream), "qex_probe_dmma_peak")
    return a.value, b.value


def declared_symbols():
    return list(_SIGNATURES)


def check(rc: int, what: str) -> None:
    if rc != QEX_OK:
        names = {1: "BAD_ARG", 2: "NOT_CONVERGED", 3: "NUMERICAL", 4: "OOM", 5: "TIMEOUT",
                 6: "CUDA_ERROR"}
        raise RuntimeError(f"{what} failed with status {rc} ({names.get(rc, '?')})")


def require_cuda():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("qex_gb300 needs a CUDA device (GB300, sm_103a); none is available")
    return torch


def ptr(t) -> int | None:
    """Device pointer of a torch tensor (or None)."""
    if t is None:
        return None
    return t.data_ptr()
