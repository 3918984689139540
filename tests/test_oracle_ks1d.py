"""CPU tests: the 1D oracle against the reference's own pins and fixtures."""

import numpy as np
import pytest

from oracle import ks1d as o


def test_xc_energy_known_answer():
    # tests/test_scf_od.py:38-62 (places=5)
    grids = np.linspace(-5, 5, 10001)
    density = np.exp(-((grids - 1) ** 2))
    e = o.xc_energy(density, o.PowerXC(-0.73855, 1 / 3), grids, "amplitude")
    assert abs(e - (-2.2660978689082367)) < 1e-5


def test_xc_potential_carries_dx():
    # tests/test_scf_od.py:64-86
    grids = np.linspace(-5, 5, 10001)
    density = np.exp(-((grids - 1) ** 2))
    v = o.xc_potential(density, o.PowerXC(-0.73855, 1 / 3), grids, "amplitude")
    np.testing.assert_allclose(v, -0.73855 * (1 / 3) * density ** (-2 / 3) * o.get_dx(grids),
                               rtol=1e-7)


@pytest.mark.parametrize("mol", ["h2", "h2_h2", "h4"])
def test_chain_potential_matches_shipped_data(golden, mol):
    ref = golden["ref"]
    grids = ref[f"{mol}_grids"]
    for loc, z, ve in zip(ref[f"{mol}_locations"], ref[f"{mol}_nuclear_charges"],
                          ref[f"{mol}_external_potentials"]):
        v = o.get_atomic_chain_potential(grids, loc, z, o.exponential_coulomb)
        np.testing.assert_allclose(v, ve, atol=1e-14, rtol=0)


def test_exact_vs_reproduces_densities_with_five_point_stencil(golden):
    ref = golden["ref"]
    grids = ref["h2_grids"]
    dx = o.get_dx(grids)
    errs = {}
    for st in (5, 3):
        e = []
        for vs, dens in zip(ref["h2_exact_v_s"], ref["h2_densities"]):
            n, _, _ = o.solve_noninteracting_system(vs, 2, grids, st)
            e.append(np.sqrt(np.sum((n - dens) ** 2) * dx))
        errs[st] = max(e)
    assert errs[5] < 3e-5  # five-point is the reference's operator
    assert errs[3] > 10 * errs[5]


def test_dense_and_banded_eigensolvers_agree():
    g = (np.arange(257) - 128) * 0.08
    v = o.get_atomic_chain_potential(g, [-1.0, 0.3, 2.0], [1, 2, 3], o.exponential_coulomb)
    for st in (3, 5):
        w1, v1 = o._lowest_eigenpairs(v, g, 5, st, "dense")
        w2, v2 = o._lowest_eigenpairs(v, g, 5, st, "banded")
        np.testing.assert_allclose(w1, w2, atol=1e-11)
        np.testing.assert_allclose(np.abs(np.sum(v1 * v2, axis=1)), 1.0, atol=1e-10)


@pytest.mark.parametrize("tol,expected", [(-1.0, [False, False, False]), (np.inf, [True, True, True])])
def test_python_driver_converged_flags(tol, expected):
    # tests/test_scf_od.py:184-215
    g = np.linspace(-5, 5, 101)
    r = o.kohn_sham([-0.5, 0.5], [1, 1], 2, 3, g, o.PowerXC(), o.exponential_coulomb, None,
                    density_mse_converge_tolerance=tol, driver="python")
    assert list(r["converged"]) == expected


@pytest.mark.parametrize("tol,expected", [(1e-2, [False, False, False]), (1e10, [False, True, True])])
def test_jit_driver_converged_flags(tol, expected):
    # tests/test_jit_scf_od.py:186-229
    g = np.linspace(-5, 5, 101)
    n0 = 2 * o.gaussian(g, 0.0, 1.0)
    r = o.kohn_sham([-0.5, 0.5], [1, 1], 2, 3, g, o.PowerXC(), o.exponential_coulomb, n0,
                    density_mse_converge_tolerance=tol, driver="jit")
    assert list(r["converged"]) == expected


@pytest.mark.parametrize("interaction", [o.soft_coulomb, o.exponential_coulomb])
def test_one_iteration_state(interaction):
    # tests/test_scf_od.py:88-142
    g = np.linspace(-5, 5, 101)
    ve = o.get_atomic_chain_potential(g, [-0.5, 0.5], [1, 1], interaction)
    n0 = 2 * o.gaussian(g, 0.0, 1.0)
    r = o.kohn_sham_iteration(n0, ve, g, 2, o.PowerXC(-0.73855, 1 / 3, 1e-10), interaction)
    assert abs(np.sum(r.density) * o.get_dx(g) - 2) < 1e-7
    assert np.isfinite(r.total_energy)
    # the dx-scaled n^(-2/3) potential of this test functional binds the two
    # lowest states at the grid edges; their splitting can round to zero
    assert r.gap >= 0


def _fd_check(xc, n, conv, reflection=False):
    g = (np.arange(n.size) - n.size // 2) * 0.08
    v = o.xc_potential(n, xc, g, conv, reflection)
    dx = o.get_dx(g)
    rng = np.random.default_rng(0)
    for i in rng.choice(n.size, 6, replace=False):
        h = 1e-6 * max(n[i], 1e-3)
        e1 = n.copy()
        e1[i] += h
        e0 = n.copy()
        e0[i] -= h
        fd = (o.xc_energy(e1, xc, g, conv, reflection) - o.xc_energy(e0, xc, g, conv, reflection)) / (2 * h)
        if conv == "local":
            fd /= dx
        assert abs(fd - v[i]) <= 1e-6 * max(1.0, abs(v[i])), (i, fd, v[i])


def test_lda_potential_matches_finite_differences():
    g = (np.arange(129) - 64) * 0.08
    n = 0.3 * np.exp(-0.5 * g ** 2) + 0.01
    _fd_check(o.LDAExpCoulomb(), n, "local")
    _fd_check(o.LDAExpCoulomb(), n, "local", reflection=True)


def test_window_mlp_potential_matches_finite_differences():
    rng = np.random.default_rng(3)
    layers = [(rng.normal(size=(17, 16)) * 0.3, rng.normal(size=16) * 0.1),
              (rng.normal(size=(16, 16)) * 0.3, rng.normal(size=16) * 0.1),
              (rng.normal(size=(16, 1)) * 0.3, rng.normal(size=1) * 0.1)]
    mlp = o.WindowMLP(layers, dtype=np.float64)
    g = (np.arange(97) - 48) * 0.08
    n = 0.4 * np.exp(-0.3 * (g - 0.5) ** 2) + 0.02
    for conv in ("local", "amplitude"):
        _fd_check(mlp, n, conv)
    _fd_check(mlp, n, "local", reflection=True)


def test_golden_oracle_fixture_is_current(golden):
    # the stored oracle outputs must match a fresh run of the oracle
    g = np.linspace(-5, 5, 101)
    n0 = 2 * o.gaussian(g, 0.0, 1.0)
    r = o.kohn_sham([-0.5, 0.5], [1, 1], 2, 4, g, o.LDAExpCoulomb(), o.exponential_coulomb, n0,
                    density_mse_converge_tolerance=-1.0, driver="jit", convention="local")
    np.testing.assert_allclose(r["total_energy"], golden["oracle"]["test_jit_energy"], rtol=1e-12)
    np.testing.assert_allclose(r["density"], golden["oracle"]["test_jit_density"], atol=1e-12)


def test_config1_converges_to_1e8():
    g = (np.arange(513) - 256) * 0.08
    ve = o.get_atomic_chain_potential(g, [-0.7, 0.7], [1, 1], o.exponential_coulomb)
    n0, _, _ = o.solve_noninteracting_system(ve, 2, g, 3, "banded")
    r = o.kohn_sham([-0.7, 0.7], [1, 1], 2, 20, g, o.LDAExpCoulomb(), o.exponential_coulomb, n0,
                    num_mixing_iterations=1, convention="local", stencil=3, method="banded")
    assert abs(r["total_energy"][-1] - r["total_energy"][-2]) < 1e-8
