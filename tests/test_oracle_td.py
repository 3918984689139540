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


def _pad(f, s, pad, idx=None):
    real = f.shape[0]
    idx = np.arange(real) if idx is None else np.asarray(idx)
    F = np.zeros((pad, pad))
    S = np.zeros((pad, pad))
    F[np.ix_(idx, idx)] = f
    S[np.ix_(idx, idx)] = s
    mask = np.zeros(pad, dtype=bool)
    mask[idx] = True
    return F, S, mask


def test_masked_eigh_reference_edge_cases():
    # tests/test_generalized_eigh_padded.py:59-172 (cases) and :280-310 (checks:
    # the lowest eigenvalue of the masked solve against the unpadded one)
    rng = np.random.default_rng(43)
    g = rng.normal(size=(3, 3))
    s_ill = np.eye(3)
    s_ill[0, 0] = 1e-8
    cases = {
        "degenerate": (np.diag([1.0, 2.0, 2.0, 3.0]), np.eye(4), 6),
        "ill_conditioned": (g @ g.T / 2, s_ill, 5),
        "negative_eigenvalues": (np.diag([-2.0, 1.0, 3.0]), np.eye(3), 5),
        "zero_eigenvalues": (np.diag([0.0, 1.0, 2.0]), np.eye(3), 5),
    }
    for name, (f, s, pad) in cases.items():
        F, S, mask = _pad(f, s, pad)
        w_ref, _ = o.generalized_eigh(f, s)
        w, v = o.masked_generalized_eigh(F, S, mask)
        assert abs(w[0] - w_ref[0]) < 1e-5, name
        np.testing.assert_allclose(w[f.shape[0]:], 0.0, atol=0)
    # the reference's slot sorting: the padded slots solve F = S = 1e-12, i.e.
    # eigenvalue 1, and the mask is applied per eigenvalue slot, so the real
    # slots hold the lowest values of the whole padded spectrum (real
    # eigenvalues above 1 are displaced); hence its checks of w[0] alone
    for name in ("degenerate", "negative_eigenvalues", "zero_eigenvalues"):
        f, s, pad = cases[name]
        real = f.shape[0]
        w, _ = o.masked_generalized_eigh(*_pad(f, s, pad))
        whole = np.sort(np.concatenate([np.diag(f), np.ones(pad - real)]))
        np.testing.assert_allclose(w[:real], whole[:real], atol=1e-12)


def test_masked_eigh_non_contiguous_mask():
    # tests/test_generalized_eigh_padded.py:176-228 and :353-384: real slots
    # 0, 2, 4 of 5; the lowest eigenvalue against the solve of the submatrices
    rng = np.random.default_rng(44)
    a, b = rng.normal(size=(3, 3)), rng.normal(size=(3, 3))
    f = a @ a.T / 2
    s = b @ b.T / 2 + 5.0 * np.eye(3)
    F, S, mask = _pad(f, s, 5, idx=[0, 2, 4])
    w_ref, _ = o.generalized_eigh(f, s)
    w, v = o.masked_generalized_eigh(F, S, mask)
    assert abs(np.sort(w)[-3:][0] - w_ref[0]) < 1e-5
    # the eigenvectors vanish on the padded basis functions
    np.testing.assert_allclose(v[~mask], 0.0, atol=0)


def test_masked_eigh_independent_of_padding_values_and_large_pad():
    # tests/test_generalized_eigh_padded.py:387-425 (padding filled with 100)
    # and :482-526 (3 real of 20)
    rng = np.random.default_rng(46)
    f, s, F, S, mask = _padded_case(rng, 3, 5)
    w1, v1 = o.masked_generalized_eigh(F, S, mask)
    F2, S2 = F.copy(), S.copy()
    F2[3:, 3:] = 100.0
    S2[3:, 3:] = 100.0
    w2, v2 = o.masked_generalized_eigh(F2, S2, mask)
    np.testing.assert_allclose(w1[:3], w2[:3], atol=1e-10)
    np.testing.assert_allclose(np.abs(v1[:3, :3]), np.abs(v2[:3, :3]), atol=1e-8)
    a, b = rng.normal(size=(3, 3)), rng.normal(size=(3, 3))
    f = (a + a.T) / 2
    s = b @ b.T / 2 + 5.0 * np.eye(3)
    F, S, mask = _pad(f, s, 20)
    w_ref, _ = o.generalized_eigh(f, s)
    w, _ = o.masked_generalized_eigh(F, S, mask)
    np.testing.assert_allclose(w[:3], w_ref, atol=1e-10)
    np.testing.assert_allclose(w[3:], 0.0, atol=0)


def _rdm1_explicit(c, occ):
    # tests/test_make_rdm1.py:10-40: C[:, occ > 0] diag(occ) C[:, occ > 0]^H
    sel = occ > 0
    return np.dot(c[:, sel] * occ[sel], c[:, sel].conj().T)


def test_make_rdm1_reference_cases():
    # tests/test_make_rdm1.py:99-193: random sizes, complex coefficients,
    # fractional occupations, hermiticity and trace
    rng = np.random.default_rng(0)
    for n, k in ((4, 2), (6, 3), (8, 4)):
        c = rng.normal(size=(n, n))
        occ = np.zeros(n)
        occ[:k] = 2.0
        np.testing.assert_allclose(o.make_rdm1(c, occ), _rdm1_explicit(c, occ), atol=1e-14)
    c = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    occ = np.array([2.0, 2.0, 0.0, 0.0])
    dm = o.make_rdm1(c, occ)
    np.testing.assert_allclose(dm, _rdm1_explicit(c, occ), atol=1e-14)
    np.testing.assert_allclose(dm, dm.conj().T, atol=1e-14)
    c = rng.normal(size=(4, 4))
    occ = np.array([1.5, 0.5, 0.0, 0.0])
    dm = o.make_rdm1(c, occ)
    np.testing.assert_allclose(dm, _rdm1_explicit(c, occ), atol=1e-14)
    q = np.linalg.qr(rng.normal(size=(4, 4)))[0]
    assert abs(np.trace(o.make_rdm1(q, np.array([2.0, 2.0, 0.0, 0.0]))) - 4.0) < 1e-12
    # unoccupied (or negative) slots do not enter
    occ = np.array([2.0, 0.0, -1.0, 0.0])
    np.testing.assert_allclose(o.make_rdm1(c, occ), 2.0 * np.outer(c[:, 0], c[:, 0]), atol=1e-14)
    # a non-finite unoccupied column (padding of a masked eigensolve) is dropped
    c_nan = c.copy()
    c_nan[:, 3] = np.nan
    c_nan[1, 2] = np.inf
    np.testing.assert_allclose(o.make_rdm1(c_nan, occ), 2.0 * np.outer(c[:, 0], c[:, 0]),
                               atol=1e-14)
