"""Fractional (Fermi-Dirac) occupations, ``qedft/train/td/fermi.py``.

CPU: the oracle on the reference tests' cases (``tests/test_fermi.py``:
electron count, monotonicity, bounds, the three variants agreeing on the
reference's spectrum, the stable variant's fallback).  GPU: the kernel
(``qex_td_fermi_occupations``, FP64) against the oracle, 1e-12 on
occupations, mu and entropic energies; the 3D SCF with Fermi occupations
against the oracle SCF (1e-8 Ha)."""

import numpy as np
import pytest

from oracle import td as o


def _cases():
    rng = np.random.default_rng(42)
    out = []
    for _ in range(20):
        n = 2 * int(rng.integers(2, 7))
        e = np.sort(rng.uniform(-5.0, 5.0, n))
        ne = 2.0 * int(rng.integers(1, n))
        theta = float(rng.uniform(0.01, 1.0))
        mu = None if rng.random() > 0.5 else float(np.mean(e) + rng.normal())
        out.append((e, ne, theta, mu))
    return out


@pytest.mark.parametrize("n_electrons", [2.0, 4.0, 6.0])
def test_oracle_reference_case(n_electrons):
    """tests/test_fermi.py:20-82 of the reference, on the oracle."""
    e = np.linspace(-1.0, 1.0, 10)
    shift = (e[2] if n_electrons == 4.0 else e[0]) + 0.9
    occ, entr, mu, loss = o.get_fractional_occupations_jax(e, n_electrons, 0.5, None, shift,
                                                           0.6, 100)
    occ0, entr0, mu0, loss0 = o.get_fractional_occupations(e, n_electrons, 1, 0.5, None, shift,
                                                           0.6, 100)
    # the early-stopping variant ends at loss < 1e-9 (|N - F| < 3e-5); the
    # reference compares the two with rtol = 1
    np.testing.assert_allclose(occ, occ0, atol=1e-4)
    assert abs(mu - mu0) < 1e-4 and abs(entr - entr0) < 1e-4
    assert abs(occ.sum() - n_electrons) < 1e-8 and loss < 1e-4
    assert np.all(np.diff(occ) <= 1e-10)


def test_oracle_stable_random_and_fallback():
    for e, ne, theta, mu in _cases():
        occ, entr, mu_f, loss = o.get_fractional_occupations_jax_stable(e, ne, theta, mu, 0.9,
                                                                        0.6, 100)
        assert abs(occ.sum() - ne) < 1e-1
        assert np.all(np.diff(occ) <= 1e-10) and occ.min() >= 0 and occ.max() <= 2
        assert loss == 0.0 and np.isfinite(entr)
    # a start so far off that Newton cannot recover: the theta = 0.01 fallback
    e = np.linspace(-1.0, 1.0, 10)
    occ, entr, mu_f, _ = o.get_fractional_occupations_jax_stable(e, 4.0, 0.001, 50.0, 0.9, 0.6, 3)
    assert abs(occ.sum() - 4.0) < 1e-1


def test_oracle_optimize_raises_when_it_fails():
    with pytest.raises(ValueError):
        o.optimize_fermi_occupations(np.array([-8.0, -4.0, 10.0]), 4.0, theta=0.04, max_steps=3)


def test_aufbau_with_fractional_remainder():
    occ, entr, _, _ = o.get_fractional_occupations(np.linspace(-1, 1, 5), 5.0, None)
    np.testing.assert_array_equal(occ, [2.0, 2.0, 1.0, 0.0, 0.0])


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def fermi():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300.td import fermi as f

    return f


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["jax", "stable"])
def test_kernel_matches_oracle(fermi, mode):
    import torch

    gpu = {"jax": fermi.get_fractional_occupations_jax,
           "stable": fermi.get_fractional_occupations_jax_stable}[mode]
    ref = {"jax": o.get_fractional_occupations_jax,
           "stable": o.get_fractional_occupations_jax_stable}[mode]
    for e, ne, theta, mu in _cases() + [(np.linspace(-1, 1, 10), 4.0, 0.5, None)]:
        shift = 0.9
        occ, entr, mu_g, loss = gpu(e, ne, theta, mu, shift, 0.6, 100)
        occ_r, entr_r, mu_r, loss_r = ref(e, ne, theta, mu, shift, 0.6, 100)
        if mode == "jax" and not loss_r < 1e-10:
            # the oracle's search did not converge: from a start just above the
            # lowest orbital the safeguarded Newton steps (up to 1e10 x the
            # gradient) go wherever rounding sends them, in the reference as
            # here, so there is nothing to compare
            continue
        np.testing.assert_allclose(occ.cpu().numpy(), occ_r, atol=1e-12, rtol=0)
        assert abs(float(mu_g) - mu_r) <= 1e-12 * max(1.0, abs(mu_r))
        assert abs(float(entr) - entr_r) <= 1e-12 * max(1.0, abs(entr_r))
        assert abs(float(loss) - loss_r) <= 1e-12 * max(1.0, abs(loss_r))
    # batched: one launch over several spectra of the same length
    es = np.stack([np.sort(np.random.default_rng(k).uniform(-3, 3, 12)) for k in range(5)])
    occ, entr, mu_g, _ = gpu(torch.as_tensor(es), torch.as_tensor([2.0, 4.0, 6.0, 8.0, 10.0]),
                             0.3, None, 0.9, 0.6, 100)
    for k in range(5):
        occ_r, entr_r, mu_r, _ = ref(es[k], 2.0 * (k + 1), 0.3, None, 0.9, 0.6, 100)
        np.testing.assert_allclose(occ[k].cpu().numpy(), occ_r, atol=1e-12, rtol=0)


@pytest.mark.gpu
def test_optimize_mode_and_failure(fermi):
    e = np.linspace(-1.0, 1.0, 10)
    occ, entr, mu, loss = fermi.get_fractional_occupations(e, 4.0, 1, 0.5, None, e[2] + 0.9,
                                                           0.6, 100)
    occ_r, entr_r, mu_r, loss_r = o.get_fractional_occupations(e, 4.0, 1, 0.5, None, e[2] + 0.9,
                                                               0.6, 100)
    np.testing.assert_allclose(occ.cpu().numpy(), occ_r, atol=1e-12, rtol=0)
    assert abs(float(loss) - loss_r) < 1e-15
    with pytest.raises(ValueError):
        fermi.optimize_fermi_occupations(np.array([-8.0, -4.0, 10.0]), 4.0, theta=0.04,
                                         max_steps=3)


@pytest.mark.gpu
def test_scf_with_fermi_occupations_matches_oracle(fermi):
    from qex_gb300.td import scf, workloads

    for na, seed, theta in ((2, 12, 0.04), (4, 14, 0.2)):
        m = workloads.synthetic_molecule(na, seed=seed)
        res = scf.run_scf(m, 12, fermi={"theta": theta})
        e_r, _, _, s_r = o.scf(m, 12, fermi={"theta": theta})
        np.testing.assert_allclose(res.energies.cpu().numpy(), e_r, atol=1e-8, rtol=0)
        np.testing.assert_allclose(res.entropic_energy.cpu().numpy(), s_r, atol=1e-10, rtol=0)
        assert abs(float(res.mo_occ.sum()) - m.nelectron) < 1e-8


@pytest.mark.gpu
def test_more_electrons_than_slots_and_bad_counts(fermi):
    """More than 2n electrons: HOMO and LUMO clamp to the highest orbital, as
    the reference's array lookup clamps them (fermi.py:422-427); a negative or
    non-finite electron count sets the molecule's status to QEX_BAD_ARG and
    leaves its neighbours in the batch untouched."""
    import torch

    from qex_gb300 import _native as N

    e = np.array([-1.0, -0.5, 0.3])
    occ, entr, mu, _ = fermi.get_fractional_occupations_jax_stable(e, 10.0, 0.1, None, 0.9,
                                                                   0.6, 100)
    occ_r, entr_r, mu_r, _ = o.get_fractional_occupations_jax_stable(e, 10.0, 0.1, None, 0.9,
                                                                     0.6, 100)
    np.testing.assert_allclose(occ.cpu().numpy(), occ_r, atol=1e-12, rtol=0)
    assert abs(float(mu) - mu_r) <= 1e-12 * max(1.0, abs(mu_r))
    es = torch.as_tensor(np.stack([e, e, e]))
    occ, entr, mu, loss, st = fermi._run(es, torch.as_tensor([2.0, -1.0, float("nan")]), 0.1,
                                         None, 0.9, 0.6, 100, 2)
    st = st.cpu().numpy()
    assert st[0] == 0 and st[1] == N.QEX_BAD_ARG and st[2] == N.QEX_BAD_ARG
    occ_r, _, _, _ = o.get_fractional_occupations_jax_stable(e, 2.0, 0.1, None, 0.9, 0.6, 100)
    np.testing.assert_allclose(occ[0].cpu().numpy(), occ_r, atol=1e-12, rtol=0)
    assert bool(torch.isnan(occ[1:]).all())
