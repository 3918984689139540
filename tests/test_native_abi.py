"""CPU tests: the C-ABI library builds, loads and exports every declared symbol."""

import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _declared():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(qex_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = _declared()
    assert "qex_ks1d_solve" in names and "qex_xc1d_eval" in names


def test_library_exports_every_declared_symbol():
    from qex_gb300 import build

    path = build.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_workspace_size_without_gpu():
    from qex_gb300 import _native as N

    lib = N.load()
    assert b"sm_103a" in lib.qex_version()
    o = N.Ks1dOptions(stencil=5, interaction=0, interaction_a=1.071295, interaction_b=1 / 2.385345,
                      num_iterations=25, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                      density_mse_converge_tolerance=-1.0, max_num_grids=513,
                      max_num_electrons=12, max_nuclei=4)
    nb = ctypes.c_size_t()
    assert lib.qex_ks1d_workspace_size(ctypes.byref(o), 4096, ctypes.byref(nb)) == 0
    assert nb.value > 4096 * 513 * 8
    o.stencil = 4
    assert lib.qex_ks1d_workspace_size(ctypes.byref(o), 4, ctypes.byref(nb)) == N.QEX_BAD_ARG
    o.stencil = 5
    o.max_num_electrons = 40  # more eigenpairs than the kernel supports
    assert lib.qex_ks1d_workspace_size(ctypes.byref(o), 4, ctypes.byref(nb)) == N.QEX_BAD_ARG
    o.max_num_electrons = 12
    # the ring's tile: 16, 32 or 64 points per chunk (0: the default); the
    # workspace holds whole chunks of any of them
    sizes = set()
    for chunk in (0, 16, 32, 64):
        o.solve_chunk = chunk
        assert lib.qex_ks1d_workspace_size(ctypes.byref(o), 8, ctypes.byref(nb)) == 0
        sizes.add(nb.value)
    assert len(sizes) == 1
    o.solve_chunk = 48
    assert lib.qex_ks1d_workspace_size(ctypes.byref(o), 8, ctypes.byref(nb)) == N.QEX_BAD_ARG


def test_ksr_workspace_adds_deferred_energy_rows_without_gpu():
    """qex_ks1d_workspace_size_xc: the base size for every functional but KSR,
    which adds num_molecules x num_iterations x max_num_grids doubles (the
    output-density rows evaluated after the SCF)."""
    from qex_gb300 import _native as N

    lib = N.load()
    o = N.Ks1dOptions(stencil=5, interaction=0, interaction_a=1.071295, interaction_b=1 / 2.385345,
                      num_iterations=15, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                      density_mse_converge_tolerance=-1.0, max_num_grids=513,
                      max_num_electrons=2, max_nuclei=2)
    base, xc_size = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.qex_ks1d_workspace_size(ctypes.byref(o), 64, ctypes.byref(base)) == 0
    spec = N.XcSpec(kind=N.QEX_XC_LDA_EXP_COULOMB)
    assert lib.qex_ks1d_workspace_size_xc(ctypes.byref(o), ctypes.byref(spec), 64,
                                          ctypes.byref(xc_size)) == 0
    assert xc_size.value == base.value
    spec = N.XcSpec(kind=N.QEX_XC_KSR, ksr_channels=16)
    assert lib.qex_ks1d_workspace_size_xc(ctypes.byref(o), ctypes.byref(spec), 64,
                                          ctypes.byref(xc_size)) == 0
    aligned = (base.value + 255) // 256 * 256
    assert xc_size.value == aligned + 8 * 64 * 15 * 513
    o.stencil = 4
    assert lib.qex_ks1d_workspace_size_xc(ctypes.byref(o), ctypes.byref(spec), 64,
                                          ctypes.byref(xc_size)) == N.QEX_BAD_ARG


def test_shell_arrays_reject_f_shells():
    import numpy as np

    from qex_gb300.td import workloads

    sh = [workloads.Shell(center=np.zeros(3), l=l, exponents=np.array([1.0]),
                          coefficients=np.array([1.0])) for l in (0, 1, 2)]
    centers, l, poff, aoff, ex, co = workloads.shell_arrays(sh)
    assert list(aoff) == [0, 1, 4] and list(poff) == [0, 1, 2, 3]
    assert workloads.cart_components(2) == [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1),
                                            (0, 0, 2)]
    sh.append(workloads.Shell(center=np.zeros(3), l=3, exponents=np.array([1.0]),
                              coefficients=np.array([1.0])))
    with pytest.raises(ValueError):
        workloads.shell_arrays(sh)


def test_numint_interface_checks_without_gpu():
    """The reference's eval_xc rule (deriv must be 1) and a neural xc_code
    without its network are rejected before any device work."""
    import numpy as np

    from qex_gb300.td.numint import NumInt

    with pytest.raises(ValueError):
        NumInt.eval_xc("LDA", np.ones(4), deriv=0)
    with pytest.raises(ValueError):
        NumInt.eval_xc("NN-LDA", np.ones(4), deriv=1)


def test_xc_resolution_rejects_arbitrary_callables():
    from qex_gb300.xc import Partial, PowerXC, resolve

    f, p = resolve(Partial(PowerXC(), params=None))
    assert isinstance(f, PowerXC)
    with pytest.raises(TypeError):
        resolve(lambda n: n)
