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


def test_xc_resolution_rejects_arbitrary_callables():
    from qex_gb300.xc import Partial, PowerXC, resolve

    f, p = resolve(Partial(PowerXC(), params=None))
    assert isinstance(f, PowerXC)
    with pytest.raises(TypeError):
        resolve(lambda n: n)
