"""CPU tests: the 3D oracle against the reference's own test semantics."""

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import td as o


def test_make_rdm1_simple_case():
    # tests/test_make_rdm1.py:85-97
    dm = o.make_rdm1(np.eye(2), np.array([2.0, 0.0]))
    np.testing.assert_allclose(dm, [[2.0, 0.0], [0.0, 0.0]], atol=1e-14)


def test_make_rdm1_trace_and_symmetry():
    rng = np.random.default_rng(0)
    c = np.linalg.qr(rng.normal(size=(8, 8)))[0]
    occ = np.array([2.0] * 4 + [0.0] * 4)
    dm = o.make_rdm1(c, occ)
    np.testing.assert_allclose(dm, dm.T, atol=1e-14)
    assert abs(np.trace(dm) - 8.0) < 1e-12


def _spd(rng, n, cond=1e3):
    q = np.linalg.qr(rng.normal(size=(n, n)))[0]
    return q @ np.diag(np.logspace(0, -np.log10(cond), n)) @ q.T


def test_generalized_eigh_matches_scipy():
    rng = np.random.default_rng(1)
    for n in (4, 17, 40):
        a = rng.normal(size=(n, n))
        a = a + a.T
        b = _spd(rng, n)
        w, v = o.generalized_eigh(a, b)
        w2 = sla.eigh(a, b, eigvals_only=True)
        np.testing.assert_allclose(w, w2, atol=1e-9 * max(1, np.abs(w2).max()))
        np.testing.assert_allclose(v.T @ b @ v, np.eye(n), atol=1e-8)


def _padded_case(rng, real, pad):
    # construction of tests/test_generalized_eigh_padded.py:15-56.  The padded
    # slots get F = S = 1e-12 on the diagonal, i.e. eigenvalue 1, and the
    # reference sorts by slot, so the physical eigenvalues must stay below 1
    # (they do for the reference's own draws); F is halved once more here so
    # that every seeded draw stays below 1 as well.
    f = rng.normal(size=(real, real))
    f = f @ f.T / 4
    s = rng.normal(size=(real, real))
    s = s @ s.T / 2 + 5.0 * np.eye(real)
    F = np.zeros((pad, pad))
    S = np.zeros((pad, pad))
    F[:real, :real] = f
    S[:real, :real] = s
    mask = np.zeros(pad, dtype=bool)
    mask[:real] = True
    return f, s, F, S, mask


@pytest.mark.parametrize("real,pad", [(3, 5), (2, 4), (1, 3), (5, 10)])
def test_masked_eigh_padding_independence(real, pad):
    # tests/test_generalized_eigh_padded.py:233-278
    rng = np.random.default_rng(real * 10 + pad)
    f, s, F, S, mask = _padded_case(rng, real, pad)
    w, v = o.generalized_eigh(f, s)
    wm, vm = o.masked_generalized_eigh(F, S, mask)
    np.testing.assert_allclose(wm[:real], w, atol=1e-10)
    np.testing.assert_allclose(wm[real:], 0.0, atol=0)
    np.testing.assert_allclose(np.abs(vm[:real, :real]), np.abs(v), atol=1e-8)
    np.testing.assert_allclose(vm[real:], 0.0, atol=0)


def test_diis_reduces_to_last_fock_below_min_vecs():
    d = o.DIIS(8, min_vecs=2)
    f = np.diag([1.0, 2.0])
    out = d.update(f, np.eye(2), np.eye(2))
    np.testing.assert_allclose(out, f)


def test_synthetic_scf_converges():
    from qex_gb300.td import workloads as W

    m = W.synthetic_molecule(3, seed=1)
    e, dm, mo = o.scf(m, max_cycle=30)
    assert abs(e[-1] - e[-2]) < 1e-8
    # electron count on the grid matches the trace of D S
    assert abs(np.trace(dm @ m.s1e) - m.nelectron) < 1e-8


def test_nn_xc_oracle_is_its_own_derivative():
    # vrho is d exc / d rho of the per-point network (the vjp with ones of
    # qedft/train/td/xc.py:12-47): central differences in FP64
    rng = np.random.default_rng(11)
    H = 24
    flat = rng.normal(0.0, 0.4, H * H + 4 * H + 1)
    rho = rng.uniform(0.0, 3.0, 80)
    exc, vrho = o.nn_xc_local(flat, rho, scale=1e-2)
    h = 1e-6
    ep, _ = o.nn_xc_local(flat, rho + h)
    em, _ = o.nn_xc_local(flat, rho - h)
    np.testing.assert_allclose((ep - em) / (2 * h), vrho, rtol=0, atol=1e-9 * np.abs(vrho).max())
    # the FP32 evaluation stays within FP32 rounding of the FP64 one
    e32, v32 = o.nn_xc_local(flat, rho, scale=1e-2, dtype=np.float32)
    np.testing.assert_allclose(e32, exc, rtol=0, atol=1e-6 * np.abs(exc).max())
    np.testing.assert_allclose(v32, vrho, rtol=0, atol=1e-5 * np.abs(vrho).max())


def test_nn_xc_global_oracle_is_its_own_derivative():
    # exc_and_vrho_global (qedft/train/td/trainer_legacy_no_jit.py:46-53): the
    # density vector is one input; vrho = d exc / d rho by central differences
    rng = np.random.default_rng(13)
    G, H = 40, 12
    flat = rng.normal(0.0, 0.3, G * H + H * H + 3 * H + 1)
    rho = rng.uniform(0.0, 2.0, G)
    exc, vrho = o.nn_xc_global(flat, rho, H)
    h = 1e-6
    fd = np.array([(o.nn_xc_global(flat, rho + h * e, H)[0] - o.nn_xc_global(flat, rho - h * e, H)[0])
                   / (2 * h) for e in np.eye(G)])
    np.testing.assert_allclose(fd, vrho, rtol=0, atol=1e-9 * np.abs(vrho).max())


def test_vwn5_correlation_known_values_and_derivative():
    # VWN paramagnetic fit 5 (the correlation of the reference's "LDA,VWN",
    # qedft/train/td/rks.py:172): eps_c(rs = 1, 2, 5) of the published fit, and
    # v_c = d(rho eps_c)/d rho
    rs = np.array([1.0, 2.0, 5.0])
    eps, _ = o.vwn5_c(3.0 / (4.0 * np.pi * rs ** 3))
    np.testing.assert_allclose(eps, [-0.0600, -0.0448, -0.0281], atol=2e-4)
    rho = np.linspace(0.01, 2.0, 30)
    h = 1e-7
    ep, _ = o.vwn5_c(rho + h)
    em, _ = o.vwn5_c(rho - h)
    _, v = o.vwn5_c(rho)
    np.testing.assert_allclose(((rho + h) * ep - (rho - h) * em) / (2 * h), v, rtol=0, atol=1e-8)
    e0, v0 = o.vwn5_c(np.zeros(3))
    assert (e0 == 0).all() and (v0 == 0).all()
