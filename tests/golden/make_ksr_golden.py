"""Generate ``tests/golden/ksr_h2.npz``: the KSR functional's fixtures.

Run from the repository root (needs the read-only reference tree):

    python tests/golden/make_ksr_golden.py <path of the reference source tree>

Stores
  * the trained global-local conv network shipped at ``data/od/h2/h2_optimal.pkl``
    (read with an unpickler that admits NumPy arrays only), as plain arrays;
  * the H2 grid and eight bond lengths of ``data/od/h2`` with their exact
    energies and densities;
  * outputs of the FP64 oracle (``oracle.ks1d.KSRGlobalConv``): eps and v_xc
    on two reference densities, and the jax_dft local-convention SCF
    (reflection symmetry, 15 iterations, one mixing step, alpha 0.5, decay
    0.9, five-point kinetic operator) at four bond lengths.
"""

from __future__ import annotations

import importlib
import pathlib
import pickle
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ks1d as o  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent
_ARRAYS_ONLY = {("numpy.core.multiarray", "_reconstruct"), ("numpy._core.multiarray", "_reconstruct"),
                ("numpy", "ndarray"), ("numpy", "dtype")}


class _ArrayUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if (module, name) not in _ARRAYS_ONLY:
            raise pickle.UnpicklingError(f"refusing {module}.{name}")
        return getattr(importlib.import_module(module.replace("numpy.core", "numpy._core")), name)


SCF_ROWS = (8, 16, 24, 40)


def main(argv):
    if len(argv) != 2:
        raise SystemExit(f"usage: python {argv[0]} <path of the reference source tree>")
    ref = pathlib.Path(argv[1])
    d = ref / "data" / "od" / "h2"
    with open(d / "h2_optimal.pkl", "rb") as fh:
        tree = _ArrayUnpickler(fh).load()
    p = o.ksr_params_from_tree(tree)
    grids = np.load(d / "grids.npy")
    rows = np.array([4, 8, 12, 16, 24, 40, 56, 71])
    out = {
        "eta": p["eta"], "w1": p["conv"][0], "w2": p["conv"][1], "w3": p["out"],
        "width": np.array(p["width"]), "grids": grids, "rows": rows,
        "distances": np.load(d / "distances.npy")[rows],
        "locations": np.load(d / "locations.npy")[rows],
        "nuclear_charges": np.load(d / "nuclear_charges.npy")[rows].astype(np.float64),
        "exact_energies": np.load(d / "total_energies.npy")[rows],
        "densities": np.load(d / "densities.npy")[rows],
    }
    xc = o.KSRGlobalConv(grids, p)
    for k in (1, 4):
        n = out["densities"][k]
        out[f"eps_{k}"] = xc.values(n)
        out[f"vxc_{k}"] = o.xc_potential(n, xc, grids, "local")
    scf_rows = [int(np.where(rows == r)[0][0]) for r in SCF_ROWS]
    out["scf_index"] = np.array(scf_rows)
    energies, finals = [], []
    for k in scf_rows:
        ve = o.get_atomic_chain_potential(grids, out["locations"][k], out["nuclear_charges"][k],
                                          o.exponential_coulomb)
        n0 = o.solve_noninteracting_system(ve, 2, grids, 5)[0]
        r = o.kohn_sham(out["locations"][k], out["nuclear_charges"][k], 2, 15, grids, xc,
                        interaction_fn=o.exponential_coulomb, initial_density=n0, alpha=0.5,
                        alpha_decay=0.9, enforce_reflection_symmetry=True,
                        num_mixing_iterations=1, convention="local", stencil=5)
        energies.append(r["total_energy"])
        finals.append(r["density"][-1])
    out["scf_total_energy"] = np.array(energies)
    out["scf_final_density"] = np.array(finals)
    np.savez_compressed(OUT / "ksr_h2.npz", **out)
    err = out["scf_total_energy"][:, -1] - out["exact_energies"][scf_rows]
    print("SCF minus exact (Ha):", err)


if __name__ == "__main__":
    main(sys.argv)
