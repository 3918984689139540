"""Training driver: datasets in jax_dft's format, the reference's loss, the
training step for L-BFGS-B, and (GPU) the adjoint of the reference's training
SCF (reflection symmetry on, energies from iteration ``ks_iter_to_ignore`` on)
against central finite differences of the FP64 oracle.

The GPU network runs in FP32; as in the differentiation test, directional
derivatives are bounded at 1e-4 relative and the loss at 1e-5 relative."""

import os

import numpy as np
import pytest

from oracle import ks1d as o


def _write_dataset(path, golden, shift=0.0):
    k = golden["ksr"]
    g = k["grids"]
    locs = k["locations"] + shift
    ve = np.array([o.get_atomic_chain_potential(g, loc, z, o.exponential_coulomb)
                   for loc, z in zip(locs, k["nuclear_charges"])])
    files = {"distances": k["distances"], "distances_x100": np.round(k["distances"] * 100),
             "grids": g, "locations": locs, "nuclear_charges": k["nuclear_charges"].astype(np.int32),
             "num_electrons": np.array(2), "total_energies": k["exact_energies"],
             "densities": k["densities"], "external_potentials": ve}
    os.makedirs(path, exist_ok=True)
    for name, arr in files.items():
        np.save(os.path.join(path, name + ".npy"), arr)
    return files


def test_dataset_format_and_selection(tmp_path, golden):
    from qex_gb300.od import train

    files = _write_dataset(tmp_path / "h2", golden)
    ds = train.Dataset(path=str(tmp_path / "h2"))
    assert ds.num_electrons == 2 and ds.grids.size == 513
    sel = [int(files["distances_x100"][i]) for i in (5, 1)]
    ms = ds.get_molecules(sel)
    np.testing.assert_array_equal(ms.distance_x100, sorted(sel))  # dataset order
    np.testing.assert_array_equal(ms.total_energy, files["total_energies"][[1, 5]])
    assert ms.density.shape == (2, 513)
    with pytest.raises(ValueError):
        ds.get_molecules([sel[0], 12345])
    cropped = train.Dataset(path=str(tmp_path / "h2"), num_grids=257)
    np.testing.assert_array_equal(cropped.grids, files["grids"][128:385])
    assert cropped.densities.shape[1] == 257
    with pytest.raises(ValueError):
        train.Dataset(path=str(tmp_path / "h2"), num_grids=256)


def test_load_molecular_datasets_checks_centering(tmp_path, golden):
    from qex_gb300.od import train

    files = _write_dataset(tmp_path / "h2", golden)
    _write_dataset(tmp_path / "h2_shifted", golden, shift=0.3)
    d = [int(files["distances_x100"][i]) for i in (1, 3)]
    out = train.load_molecular_datasets(["h2"], {"dataset1": d}, base_path=tmp_path)
    assert len(out) == 1 and out[0][1].locations.shape == (2, 2)
    with pytest.raises(ValueError):
        train.load_molecular_datasets(["h2_shifted"], {"dataset1": d}, base_path=tmp_path)
    with pytest.raises(RuntimeError):
        train.load_molecular_datasets(["missing"], {"dataset1": d}, base_path=tmp_path)


def test_flatten_roundtrip():
    from qex_gb300.od import train

    rng = np.random.default_rng(0)
    params = [(rng.normal(size=(17, 16)), rng.normal(size=16)),
              (rng.normal(size=(16, 1)), rng.normal(size=1))]
    spec, flat = train.flatten(params)
    assert flat.size == 17 * 16 + 16 + 16 + 1
    back = train.unflatten(spec, flat)
    for (a, b), (c, d) in zip(params, back):
        np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(b, d)
    with pytest.raises(ValueError):
        train.unflatten(spec, flat[:-1])


def test_trajectory_loss_matches_oracle_and_its_gradients():
    import torch

    from qex_gb300.od.adjoint import TrajectoryLoss

    rng = np.random.default_rng(1)
    B, T, N = 3, 15, 33
    g = (np.arange(N) - 16) * 0.08
    e = rng.normal(-1.5, 0.1, (B, T))
    te = rng.normal(-1.5, 0.1, B)
    nf, tn = rng.random((B, N)), rng.random((B, N))
    ne = 2
    loss = TrajectoryLoss(0.9, 10)
    t = lambda a: torch.as_tensor(np.asarray(a, np.float64))  # noqa: E731
    dx = t(np.full(B * N, 0.08))
    ne_b, ne_p = t(np.full(B, ne)), t(np.full(B * N, ne))
    val = loss.value(t(e), t(nf.ravel()), t(te), t(tn.ravel()), dx, ne_b, ne_p)
    ref = o.reference_training_loss(e, nf, te, tn, g, ne, 0.9, 10)
    assert abs(val - ref) < 1e-13 * max(1.0, abs(ref))
    h = 1e-6
    for tt in (9, 10, 12, 14):
        ge = loss.grad_energy(tt, t(e), t(te), ne_b)
        if tt < 10:
            assert ge is None
            continue
        for b in range(B):
            ep, em = e.copy(), e.copy()
            ep[b, tt] += h
            em[b, tt] -= h
            fd = (o.reference_training_loss(ep, nf, te, tn, g, ne, 0.9, 10)
                  - o.reference_training_loss(em, nf, te, tn, g, ne, 0.9, 10)) / (2 * h)
            assert abs(float(ge[b]) - fd) < 1e-7
    gd = loss.grad_density(t(nf.ravel()), t(tn.ravel()), dx, ne_p, B).numpy().reshape(B, N)
    for b, i in ((0, 3), (2, 20)):
        fp, fm = nf.copy(), nf.copy()
        fp[b, i] += h
        fm[b, i] -= h
        fd = (o.reference_training_loss(e, fp, te, tn, g, ne, 0.9, 10)
              - o.reference_training_loss(e, fm, te, tn, g, ne, 0.9, 10)) / (2 * h)
        assert abs(gd[b, i] - fd) < 1e-8


def test_training_step_and_lbfgs_plumbing(tmp_path):
    """create_training_step with a quadratic stand-in for the SCF adjoint:
    records, checkpoints and drives scipy's L-BFGS-B to the minimum."""
    import pickle

    import scipy.optimize

    from qex_gb300.od import train

    target = np.linspace(-1, 1, 7)

    def vg(flat, locations, nuclear_charges, initial_density, target_energy, target_density):
        d = np.asarray(flat) - target
        return float(d @ d), 2 * d

    ts = train.MoleculeSet(np.zeros((1, 2)), np.ones((1, 2)), np.zeros(1), np.zeros((1, 5)),
                           np.zeros((1, 5)), np.array([100]), np.linspace(-1, 1, 5), 2)
    spec = [((7,), (0,))]
    step = train.create_training_step(vg, ts, None, save_every_n=2, checkpoint_dir=str(tmp_path),
                                      spec=spec, ckpt_prefix="ck")
    x, f, info = scipy.optimize.fmin_l_bfgs_b(step, x0=np.zeros(7), maxiter=50)
    np.testing.assert_allclose(x, target, atol=1e-6)
    assert step.loss_record[0] > step.loss_record[-1]
    with open(tmp_path / "ck-00000", "rb") as fh:
        w, b = pickle.load(fh)[0]
    np.testing.assert_array_equal(w, np.zeros(7))


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _oracle_train_loss(mols, flat, T, te, tn, ignore, discount):
    from qex_gb300.xc import WindowMLPFunctional

    layers = WindowMLPFunctional.unflatten(flat, np.float64)
    xc = o.WindowMLP([(np.asarray(a, np.float64), np.asarray(b, np.float64)) for a, b in layers],
                     dtype=np.float64)
    total, B = 0.0, len(mols)
    for (n, r, z, ne), e_t, n_t in zip(mols, te, tn):
        g = (np.arange(n) - (n - 1) / 2) * 0.08
        ve = o.get_atomic_chain_potential(g, r, z, o.exponential_coulomb)
        n0, _, _ = o.solve_noninteracting_system(ve, ne, g, 5, "banded")
        res = o.kohn_sham(r, z, ne, T, g, xc, o.exponential_coulomb, n0, alpha=0.5,
                          alpha_decay=0.9, num_mixing_iterations=1, convention="local",
                          stencil=5, method="banded", enforce_reflection_symmetry=True)
        # per-molecule terms of the batch mean
        total += o.reference_training_loss(res["total_energy"][None, :], res["density"][-1][None],
                                           np.array([e_t]), n_t[None], g, ne, discount, ignore)
    return total / B


@pytest.mark.gpu
def test_reference_loss_adjoint_with_reflection_matches_finite_differences():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300 import networks
    from qex_gb300.od import adjoint, engine as eng
    from qex_gb300.xc import Partial, WindowMLPFunctional

    mols = [(129, [-0.6, 0.6], [1.0, 1.0], 2), (161, [-1.2, 0.3], [1.0, 2.0], 3),
            (129, [-0.9, 0.9], [1.0, 1.0], 2)]
    T, ignore, disc = 12, 8, 0.9
    init_fn, xc_fn = networks.build_xc_functional(networks.WindowMLP().build_network(None),
                                                  np.zeros(5))
    params = init_fn(5)
    flat = WindowMLPFunctional.flatten(params).astype(np.float64)
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
                          convention="local", stencil=5, enforce_reflection_symmetry=True)
    res = adjoint.Ks1dAdjoint().value_and_grad(
        batch, Partial(xc_fn, params=params), cfg, te, np.concatenate(tn), checkpoint_every=5,
        loss=adjoint.TrajectoryLoss(disc, ignore))
    loss_ref = _oracle_train_loss(mols, flat, T, te, tn, ignore, disc)
    assert abs(res.loss - loss_ref) <= 1e-5 * max(1.0, abs(loss_ref))
    rng = np.random.default_rng(2)
    h = 1e-5
    for trial in range(3):
        d = rng.normal(size=flat.size)
        d /= np.linalg.norm(d)
        fd = (_oracle_train_loss(mols, flat + h * d, T, te, tn, ignore, disc)
              - _oracle_train_loss(mols, flat - h * d, T, te, tn, ignore, disc)) / (2 * h)
        ad = float(res.grad @ d)
        assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.linalg.norm(res.grad)), (trial, ad, fd)


@pytest.mark.gpu
def test_lbfgs_training_on_h2_reduces_the_loss(golden, tmp_path):
    """The reference's training loop (trainer.py:150-178) on two H2 bond lengths
    of data/od/h2 (exact energies and densities as targets), a few L-BFGS-B
    iterations of the window MLP."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qex_gb300 import networks
    from qex_gb300.od import train

    files = _write_dataset(tmp_path / "h2", golden)
    sel = [int(files["distances_x100"][i]) for i in (1, 3)]
    (ds, ts), = train.load_molecular_datasets(["h2"], {"dataset1": sel}, base_path=tmp_path)
    init_fn, xc_fn = networks.build_xc_functional(networks.WindowMLP().build_network(None),
                                                  ds.grids)
    params, loss, info = train.train(xc_fn, init_fn(0), ts,
                                     {"maxiter": 3, "maxfun": 6, "save_every_n": 100})
    rec = info["loss_record"]
    assert len(rec) >= 2 and np.isfinite(rec).all()
    assert min(rec[1:]) < rec[0]
