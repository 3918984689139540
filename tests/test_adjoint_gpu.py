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


def test_custom_vjp_pair_matches_value_and_grad_and_fd():
    """scf_fwd / scf_bwd in the jax.custom_vjp calling convention: with the
    loss's cotangents the gradient equals value_and_grad's (bitwise); with an
    arbitrary cotangent on the energy trajectory and the final density, the
    vector-Jacobian product matches central differences of the same GPU
    forward (FP64 network) to 1e-6."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300 import networks
    from qex_gb300.od import adjoint, engine as eng
    from qex_gb300.xc import Partial, WindowMLPFunctional

    rng = np.random.default_rng(4)
    ms = [eng.Molecule1D(num_grids=161, grid_spacing=0.08, locations=[-r / 2, r / 2],
                         nuclear_charges=[1.0, 1.0], num_electrons=2)
          for r in rng.uniform(0.8, 2.5, 3)]
    batch = eng.PackedBatch(ms, sort=False)
    cfg = eng.SolveConfig(num_iterations=7, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                          convention="local", stencil=5)
    init_fn, _ = networks.build_xc_functional(networks.WindowMLP().build_network(None),
                                              np.zeros(5))
    flat = WindowMLPFunctional.flatten(init_fn(2)).astype(np.float64)
    f64 = WindowMLPFunctional(2.0, precision="fp64")

    def xc_of(v):
        return Partial(f64, params=WindowMLPFunctional.unflatten(v, np.float64))

    (E, n), res = adjoint.scf_fwd(xc_of(flat), batch, cfg, checkpoint_every=3)
    gE = torch.as_tensor(rng.normal(size=tuple(E.shape)), device="cuda")
    gN = torch.as_tensor(rng.normal(size=n.numel()) * 1e-2, device="cuda")
    g = adjoint.scf_bwd(res, (gE, gN))

    def objective(v):
        (e, d), _ = adjoint.scf_fwd(xc_of(v), batch, cfg, checkpoint_every=3)
        return float((gE * e).sum() + (gN * d).sum())

    h = 1e-5
    d = rng.normal(size=flat.size)
    d /= np.linalg.norm(d)
    fd = (objective(flat + h * d) - objective(flat - h * d)) / (2 * h)
    assert abs(g @ d - fd) <= 1e-6 * abs(fd), (g @ d, fd)
    # the loss's cotangents reproduce value_and_grad
    te = np.full(3, -1.0)
    tn = np.zeros(n.numel())
    vg = adjoint.Ks1dAdjoint().value_and_grad(batch, xc_of(flat), cfg, te, tn, checkpoint_every=3)
    loss = adjoint.Config3Loss(0.1)
    dx = torch.full_like(n, 0.08)
    g_e = torch.zeros_like(E)
    g_e[:, -1] = 2.0 * (E[:, -1] - torch.as_tensor(te, device="cuda"))
    g_n = loss.grad_density(n, torch.as_tensor(tn, device="cuda"), dx, None, 3)
    np.testing.assert_array_equal(adjoint.scf_bwd(res, (g_e, g_n)), vg.grad)
