"""Molecular integration grids (pyscf gen_grid.Grids with becke_scheme =
stratmann, as the reference builds them): CPU checks of the oracle's radial
and angular rules and of multi-centre integrals against closed forms; GPU
parity of the partition kernel with the oracle (1e-10 relative)."""

import math

import numpy as np
import pytest

from oracle import td as o


def _gauss_pair(c, w, A, B, a, b):
    """Numerical and analytic int exp(-a|r-A|^2) exp(-b|r-B|^2) d^3r."""
    f = np.exp(-a * ((c - A) ** 2).sum(1) - b * ((c - B) ** 2).sum(1))
    exact = (math.pi / (a + b)) ** 1.5 * math.exp(-a * b / (a + b) * ((A - B) ** 2).sum())
    return float(np.dot(w, f)), exact


def test_radial_and_angular_rules():
    r, w = o.radial_m4(50, 0.8)
    assert abs(4 * math.pi * np.dot(w, np.exp(-r * r)) - math.pi ** 1.5) < 1e-12
    u, wa = o.angular_rule(12)
    assert abs(wa.sum() - 4 * math.pi) < 1e-12
    x, y, z = u.T
    # int x^2 = int z^2 = 4 pi / 3, odd moments vanish, int z^4 = 4 pi / 5
    assert abs(np.dot(wa, x * x) - 4 * math.pi / 3) < 1e-12
    assert abs(np.dot(wa, z ** 4) - 4 * math.pi / 5) < 1e-12
    assert abs(np.dot(wa, x * y * z)) < 1e-12


@pytest.mark.parametrize("scheme", ["stratmann", "becke"])
def test_multicentre_gaussian_integrals(scheme):
    from qex_gb300.td import workloads

    m = workloads.synthetic_molecule(4, seed=14, with_integrals=False)
    c, w = o.becke_grid(m.charges, m.positions, 3, scheme)
    P = m.positions
    for (i, j), (a, b) in (((0, 1), (0.4, 0.7)), ((1, 2), (1.5, 0.9)), ((0, 3), (0.3, 0.3))):
        num, exact = _gauss_pair(c, w, P[i], P[j], a, b)
        # error measured against the integrand's scale (pi/(a+b))^(3/2): the
        # overlap factor can make the integral itself tiny
        assert abs(num - exact) <= 1e-5 * (math.pi / (a + b)) ** 1.5, (i, j, num, exact)


def test_host_tables_match_oracle():
    from qex_gb300.td import grids

    for n, xi in ((30, 0.8), (75, 1.1)):
        r, w = grids.treutler_ahlrichs(n, xi)
        r_o, w_o = o.radial_m4(n, xi)
        # log((1 - x) / 2) and -log(2 / (1 - x)) round differently near r = 0
        np.testing.assert_allclose(r, r_o, rtol=1e-11)
        np.testing.assert_allclose(w, w_o, rtol=1e-11)
    u, wa = grids.angular_product(10)
    u_o, wa_o = o.angular_rule(10)
    np.testing.assert_allclose(u, u_o, atol=1e-15)
    np.testing.assert_allclose(wa, wa_o, rtol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["stratmann", "becke"])
def test_grid_kernel_matches_oracle(scheme):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300.td import grids, workloads

    for na, seed, level in ((1, 11, 2), (4, 14, 3), (8, 18, 2)):
        m = workloads.synthetic_molecule(na, seed=seed, with_integrals=False)
        g = grids.Grids(m)
        g.level = level
        g.becke_scheme = grids.stratmann if scheme == "stratmann" else grids.original_becke
        g.build()
        c_o, w_o = o.becke_grid(m.charges, m.positions, level, scheme)
        # the host radial tables and the oracle's differ at 1e-12 relative
        np.testing.assert_allclose(g.coords.cpu().numpy(), c_o, atol=1e-10, rtol=0)
        np.testing.assert_allclose(g.weights.cpu().numpy(), w_o, rtol=1e-10,
                                   atol=1e-13 * float(np.abs(w_o).max()))


@pytest.mark.gpu
def test_becke_molecule_integrates_the_density():
    """On a Becke grid the synthetic model's quadratures become accurate: the
    SCF density integrates to the electron count."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300.td import numint, scf, workloads

    m = workloads.synthetic_molecule(3, seed=13, grid="becke", level=3)
    res = scf.run_scf(m, 15)
    nelec, _, _ = numint.nr_rks(m.ao, m.weights, res.dm)
    assert abs(float(nelec) - m.nelectron) < 1e-6
