"""Generate the committed golden fixtures for the 1D Kohn-Sham tests.

Run from the repository root (needs the read-only reference tree):

    python tests/golden/make_golden.py <path of the reference source tree>

Writes ``tests/golden/ks1d_reference_data.npz`` (small slices of the
reference's shipped datasets, ``data/od/{h2,h2_h2,h4}``) and
``tests/golden/ks1d_oracle.npz`` (outputs of the NumPy oracle on fixed cases,
so the GPU tests have stored expected values).
"""

from __future__ import annotations

import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ks1d as o  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent


def reference_slices(ref: pathlib.Path):
    data = {}
    for mol in ("h2", "h2_h2", "h4"):
        d = ref / "data" / "od" / mol
        rows = np.linspace(0, len(np.load(d / "distances.npy")) - 1, 4).astype(int)
        data[f"{mol}_grids"] = np.load(d / "grids.npy")
        data[f"{mol}_locations"] = np.load(d / "locations.npy")[rows]
        data[f"{mol}_nuclear_charges"] = np.load(d / "nuclear_charges.npy")[rows].astype(np.float64)
        data[f"{mol}_external_potentials"] = np.load(d / "external_potentials.npy")[rows]
        data[f"{mol}_num_electrons"] = np.array(int(np.load(d / "num_electrons.npy")))
        if mol == "h2":
            data["h2_exact_v_s"] = np.load(d / "exact_v_s.npy")[rows]
            data["h2_densities"] = np.load(d / "densities.npy")[rows]
    return data


def oracle_cases():
    out = {}
    # config-1 shape: 513 points, dx 0.08, H2 at +-0.7, exp-Coulomb LDA, 20 iterations
    g = (np.arange(513) - 256) * 0.08
    lda = o.LDAExpCoulomb()
    ve = o.get_atomic_chain_potential(g, [-0.7, 0.7], [1, 1], o.exponential_coulomb)
    for st in (3, 5):
        n0, _, _ = o.solve_noninteracting_system(ve, 2, g, st)
        r = o.kohn_sham([-0.7, 0.7], [1, 1], 2, 20, g, lda, o.exponential_coulomb, n0, alpha=0.5,
                        alpha_decay=0.9, num_mixing_iterations=1, convention="local", stencil=st)
        out[f"h2_lda_st{st}_initial_density"] = n0
        out[f"h2_lda_st{st}_total_energy"] = r["total_energy"]
        out[f"h2_lda_st{st}_density"] = r["density"][-1]
        out[f"h2_lda_st{st}_gap"] = r["gap"]
    # the reference tests' system (101 points on [-5,5], H2 at +-0.5, Gaussian
    # start) with the LDA: the power functional of those tests binds two
    # degenerate edge states, which leaves the output density undetermined
    g = np.linspace(-5, 5, 101)
    n0 = 2 * o.gaussian(g, 0.0, 1.0)
    r = o.kohn_sham([-0.5, 0.5], [1, 1], 2, 4, g, o.LDAExpCoulomb(), o.exponential_coulomb, n0,
                    density_mse_converge_tolerance=-1.0, driver="jit", convention="local")
    out["test_jit_energy"] = r["total_energy"]
    out["test_jit_density"] = r["density"]
    out["test_jit_converged"] = r["converged"]
    return out


def main(argv):
    if len(argv) != 2:
        raise SystemExit(f"usage: python {argv[0]} <path of the reference source tree>")
    ref = pathlib.Path(argv[1])
    np.savez_compressed(OUT / "ks1d_reference_data.npz", **reference_slices(ref))
    np.savez_compressed(OUT / "ks1d_oracle.npz", **oracle_cases())
    print("wrote", OUT / "ks1d_reference_data.npz", OUT / "ks1d_oracle.npz")


if __name__ == "__main__":
    main(sys.argv)
