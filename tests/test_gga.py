"""GGA numint (the GGA branch of qedft/train/td/numint_legacy.py:175-198):
AO gradients, rho and grad rho, PBE exchange, the GGA potential matrix and
the SCF with it.  CPU: the oracle against finite differences.  GPU: the
kernels against the oracle (FP64: 1e-12 on values, 1e-10 on matrices,
1e-8 Ha on SCF energies).  PBE exchange is restated from its publication
(libxc is not available, so its parity is against the restatement)."""

import numpy as np
import pytest

from oracle import td as o


def _mol(na=2, seed=12):
    from qex_gb300.td import workloads

    return workloads.synthetic_molecule(na, seed=seed)


def _ao4(m, coords=None):
    a = o.eval_ao(m.shells, m.coords if coords is None else coords, deriv=1)
    return np.concatenate([a[0][None], a[1]], axis=0)


def test_pbe_x_derivatives():
    rng = np.random.default_rng(0)
    r, s = rng.uniform(1e-3, 3.0, 50), rng.uniform(0.0, 5.0, 50)
    _, vr, vs = o.pbe_x(r, s)
    e = lambda a, b: o.pbe_x(a, b)[0] * a  # noqa: E731
    h = 1e-7
    np.testing.assert_allclose((e(r + h, s) - e(r - h, s)) / (2 * h), vr, atol=1e-8, rtol=1e-6)
    np.testing.assert_allclose((e(r, s + h) - e(r, s - h)) / (2 * h), vs, atol=1e-8, rtol=1e-6)
    # uniform density: PBE reduces to the Slater exchange
    np.testing.assert_allclose(o.pbe_x(r, 0.0 * s)[0], o.lda_x(r)[0], rtol=1e-14)


def test_ao_gradient_and_gga_vmat_finite_differences():
    m = _mol()
    ao4 = _ao4(m)
    h = 1e-6
    for d in range(3):
        dc = np.zeros(3)
        dc[d] = h
        fd = (o.eval_ao(m.shells, m.coords + dc) - o.eval_ao(m.shells, m.coords - dc)) / (2 * h)
        np.testing.assert_allclose(ao4[1 + d], fd, atol=1e-7)
    e0, c0 = o.generalized_eigh(m.h1e, m.s1e)
    dm = o.make_rdm1(c0, o.get_occ(m.nelectron, e0))
    _, exc, vmat = o.nr_rks_gga(ao4, m.weights, dm)
    for i, j in ((0, 0), (1, 3), (2, 5)):
        dd = np.zeros_like(dm)
        dd[i, j] += 1.0
        dd[j, i] += 1.0
        ep = o.nr_rks_gga(ao4, m.weights, dm + 1e-6 * dd)[1]
        em = o.nr_rks_gga(ao4, m.weights, dm - 1e-6 * dd)[1]
        assert abs((ep - em) / 2e-6 - (vmat[i, j] + vmat[j, i])) < 1e-6


@pytest.fixture(scope="module")
def td():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300.td import numint, scf

    return numint, scf


@pytest.mark.gpu
def test_gga_kernels_match_oracle(td):
    numint, _ = td
    for na, seed in ((2, 12), (8, 18)):
        m = _mol(na, seed)
        ao4_r = _ao4(m)
        ao4 = numint.eval_ao_deriv1(m)
        np.testing.assert_allclose(ao4.cpu().numpy(), ao4_r, atol=1e-13, rtol=0)
        e0, c0 = o.generalized_eigh(m.h1e, m.s1e)
        dm = o.make_rdm1(c0, o.get_occ(m.nelectron, e0))
        rho4 = numint.eval_rho_gga(ao4, dm)
        np.testing.assert_allclose(rho4.cpu().numpy(), o.eval_rho_gga(ao4_r, dm), atol=1e-12,
                                   rtol=0)
        nelec, excsum, vmat = numint.nr_rks(ao4, m.weights, dm, "PBE_X")
        n_r, e_r, v_r = o.nr_rks_gga(ao4_r, m.weights, dm)
        assert abs(float(nelec) - n_r) < 1e-10 and abs(float(excsum) - e_r) < 1e-10
        np.testing.assert_allclose(vmat.cpu().numpy(), v_r, atol=1e-10, rtol=0)


@pytest.mark.gpu
def test_gga_scf_matches_oracle(td):
    _, scf = td
    for na, seed in ((2, 12), (4, 14)):
        m = _mol(na, seed)
        res = scf.run_scf(m, 12, xc="PBE_X")
        e_r, _, _ = o.scf(m, 12, gga=True)
        np.testing.assert_allclose(res.energies.cpu().numpy(), e_r, atol=1e-8, rtol=0)
