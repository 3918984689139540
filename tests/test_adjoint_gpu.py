"""GPU test of the hand-written SCF adjoint against central finite differences
of the FP64 oracle (the same network parameters evaluated in FP64, perturbed
in FP64, h = 1e-5).

The GPU network runs in FP32, so the function it differentiates differs from
the oracle's FP64 network by FP32 rounding; the directional-derivative bound
is 1e-4 relative.  The adjoint equations themselves agree with central
differences to ~3e-8 when evaluated entirely in FP64."""

import numpy as np
import pytest

from oracle import ks1d as o

pytestmark = pytest.mark.gpu


def _oracle_loss(mols, flat, T, target_e, target_n, w, dx=0.08):
    from qex_gb300.xc import WindowMLPFunctional

    layers = WindowMLPFunctional.unflatten(flat, np.float64)
    xc = o.WindowMLP([(np.asarray(a, np.float64), np.asarray(b, np.float64)) for a, b in layers],
                     dtype=np.float64)
    loss = 0.0
    for (n, r, z, ne), te, tn in zip(mols, target_e, target_n):
        g = (np.arange(n) - (n - 1) / 2) * dx
        ve = o.get_atomic_chain_potential(g, r, z, o.exponential_coulomb)
        n0, _, _ = o.solve_noninteracting_system(ve, ne, g, 5, "banded")
        res = o.kohn_sham(r, z, ne, T, g, xc, o.exponential_coulomb, n0, alpha=0.5,
                          alpha_decay=0.9, num_mixing_iterations=1, convention="local",
                          stencil=5, method="banded")
        loss += (res["total_energy"][-1] - te) ** 2 + w * np.sum((res["density"][-1] - tn) ** 2) * dx
    return loss


def test_adjoint_matches_finite_differences():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300 import networks
    from qex_gb300.od import adjoint, engine as eng
    from qex_gb300.xc import Partial, WindowMLPFunctional

    mols = [(129, [-0.6, 0.6], [1.0, 1.0], 2), (161, [-1.2, 0.3], [1.0, 2.0], 3),
            (129, [-0.9, 0.9], [1.0, 1.0], 2)]
    T, w = 6, 0.1
    init_fn, xc_fn = networks.build_xc_functional(networks.WindowMLP().build_network(None),
                                                  np.zeros(5))
    params = init_fn(3)
    flat = WindowMLPFunctional.flatten(params).astype(np.float64)
    # targets: the plain LDA solve (as in the differentiation configuration)
    te, tn = [], []
    for n, r, z, ne in mols:
        g = (np.arange(n) - (n - 1) / 2) * 0.08
        ve = o.get_atomic_chain_potential(g, r, z, o.exponential_coulomb)
        n0, _, _ = o.solve_noninteracting_system(ve, ne, g, 5, "banded")
        res = o.kohn_sham(r, z, ne, T, g, o.LDAExpCoulomb(), o.exponential_coulomb, n0,
                          num_mixing_iterations=1, convention="local", method="banded")
        te.append(res["total_energy"][-1])
        tn.append(res["density"][-1])
    ms = [eng.Molecule1D(num_grids=n, grid_spacing=0.08, locations=r, nuclear_charges=z,
                         num_electrons=ne) for n, r, z, ne in mols]
    batch = eng.PackedBatch(ms, sort=False)
    cfg = eng.SolveConfig(num_iterations=T, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                          convention="local", stencil=5)
    adj = adjoint.Ks1dAdjoint()
    res = adj.value_and_grad(batch, Partial(xc_fn, params=params), cfg, te,
                             np.concatenate(tn), density_weight=w, checkpoint_every=4)
    loss_ref = _oracle_loss(mols, flat, T, te, tn, w)
    assert abs(res.loss - loss_ref) <= 1e-5 * max(1.0, abs(loss_ref))
    rng = np.random.default_rng(0)
    h = 1e-5
    for trial in range(3):
        d = rng.normal(size=flat.size)
        d /= np.linalg.norm(d)
        fd = (_oracle_loss(mols, flat + h * d, T, te, tn, w)
              - _oracle_loss(mols, flat - h * d, T, te, tn, w)) / (2 * h)
        ad = float(res.grad @ d)
        assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.linalg.norm(res.grad)), (trial, ad, fd)


def test_adjoint_fp64_network_matches_central_differences_at_1e6():
    """The differentiation configuration's check at its shape: H2-type
    molecules (unit charges, separation uniform in [0.5, 3.0] bohr) on 513
    points, 15 unrolled iterations, checkpoints every 5, the loss
    sum (E - E_t)^2 + 0.1 sum |n - n_t|^2 dx with targets from the plain LDA
    solve.  With the network in FP64 (the checking mode of the window MLP),
    the hand-written adjoint matches central finite differences of the FP64
    oracle (h = 1e-5) to 1e-6 relative along random directions."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300 import networks
    from qex_gb300.od import adjoint, engine as eng
    from qex_gb300.xc import Partial, WindowMLPFunctional

    rng = np.random.default_rng(2024)
    B, n, T, w = 8, 513, 15, 0.1
    mols = []
    for R in rng.uniform(0.5, 3.0, B):
        mols.append((n, [-R / 2, R / 2], [1.0, 1.0], 2))
    init_fn, _ = networks.build_xc_functional(networks.WindowMLP().build_network(None),
                                              np.zeros(5))
    params32 = init_fn(9)
    flat = WindowMLPFunctional.flatten(params32).astype(np.float64)
    te, tn = [], []
    for nn_, r, z, ne in mols:
        g = (np.arange(nn_) - (nn_ - 1) / 2) * 0.08
        ve = o.get_atomic_chain_potential(g, r, z, o.exponential_coulomb)
        n0, _, _ = o.solve_noninteracting_system(ve, ne, g, 5, "banded")
        res = o.kohn_sham(r, z, ne, T, g, o.LDAExpCoulomb(), o.exponential_coulomb, n0,
                          num_mixing_iterations=1, convention="local", method="banded")
        te.append(res["total_energy"][-1])
        tn.append(res["density"][-1])
    ms = [eng.Molecule1D(num_grids=nn_, grid_spacing=0.08, locations=r, nuclear_charges=z,
                         num_electrons=ne) for nn_, r, z, ne in mols]
    batch = eng.PackedBatch(ms, sort=False)
    cfg = eng.SolveConfig(num_iterations=T, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                          convention="local", stencil=5)
    f64 = WindowMLPFunctional(2.0, precision="fp64")
    params64 = WindowMLPFunctional.unflatten(flat, np.float64)
    res = adjoint.Ks1dAdjoint().value_and_grad(batch, Partial(f64, params=params64), cfg, te,
                                               np.concatenate(tn), density_weight=w,
                                               checkpoint_every=5)
    loss_ref = _oracle_loss(mols, flat, T, te, tn, w)
    assert abs(res.loss - loss_ref) <= 1e-9 * max(1.0, abs(loss_ref)), (res.loss, loss_ref)
    h = 1e-5
    for trial in range(3):
        d = rng.normal(size=flat.size)
        d /= np.linalg.norm(d)
        fd = (_oracle_loss(mols, flat + h * d, T, te, tn, w)
              - _oracle_loss(mols, flat - h * d, T, te, tn, w)) / (2 * h)
        ad = float(res.grad @ d)
        assert abs(ad - fd) <= 1e-6 * abs(fd), (trial, ad, fd, abs(ad - fd) / abs(fd))
