"""The reference's dense XC networks on the GPU path: LocalMLP and GlobalMLP
(``qedft/models/networks.py:83-138``) with the wrappers of
``qedft/models/wrappers.py:162-217`` (self-interaction layer, negativity
transform, the global mean), through ``build_xc_functional`` into both SCF
conventions.

CPU: the oracle's potentials against finite differences of its energies, the
packed device layout, the wrapper parameter trees and the interface checks.
GPU: the standalone evaluation and the SCF (the amplitude-encoded scan of
``qedft/train/od/jit_scf.py:247-330`` for GlobalMLP, jax_dft ``kohn_sham``
for LocalMLP) against the oracle with the same FP32 network arithmetic.
The networks run in FP32 on the GPU, so the bounds are those of FP32
rounding: 2e-6 relative on E_xc, 1e-5 on v_xc, 2e-6 Ha on SCF energies and
1e-6 L2 on densities.
"""

import numpy as np
import pytest

from oracle import ks1d as o


def _grids(n):
    return (np.arange(n) - (n - 1) / 2) * 0.08


def _density(g, r=0.7):
    n = np.exp(-(g - r) ** 2) + np.exp(-(g + r) ** 2)
    return 2.0 * n / (np.sum(n) * 0.08)


def _oracle_xc(functional, params, grids, dtype=np.float32):
    layers, width = functional.dense_layers(params)
    return o.DenseNetworkXC(grids, layers, functional.activation, functional.normalization,
                            functional.local, functional.self_interaction,
                            functional.negativity, width, dtype=dtype)


def _build(kind, grids, **cfg):
    from qex_gb300 import networks

    net_cls = networks.LocalMLP if kind == "local" else networks.GlobalMLP
    net = net_cls(cfg)
    init_fn, xc_fn = networks.build_xc_functional(net.build_network(grids), grids, net.config)
    return init_fn, xc_fn


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("local", [True, False])
@pytest.mark.parametrize("si", [False, True])
def test_oracle_potential_matches_finite_differences(local, si):
    from qex_gb300 import networks

    g = _grids(65)
    n = _density(g)
    rng = np.random.default_rng(1)
    for act in ("tanh", "gelu", "softplus", "selu"):
        layers = [p for p in networks.dense_stack_params(2, 1 if local else g.size, 12, 3) if p]
        xc = o.DenseNetworkXC(g, layers, act, 2.0, local, si, True, 0.8)
        cot = rng.normal(size=g.size)
        d = rng.normal(size=g.size)
        h = 1e-6
        fd = (cot @ xc.values(n + h * d) - cot @ xc.values(n - h * d)) / (2 * h)
        assert abs(fd - xc.vjp(n, cot) @ d) <= 1e-6 * abs(fd)


def test_wrapper_trees_and_packed_layout():
    """The wrapped parameter trees nest as the reference's stax combinators
    do (negativity: [net, ()]; self-interaction: [(), ((), net), (width,)]),
    and the device layout pads the hidden width to a multiple of 8 with zeros."""
    g = _grids(33)
    init_fn, xc_fn = _build("global", g, n_neurons=12, n_layers=2)
    params = init_fn(0)
    assert params[1] == () and params[0][0] == () and params[0][2][0] == 1.0
    f = xc_fn.functional
    assert f.self_interaction and f.negativity and not f.local and f.num_inputs == 33
    layers, width = f.dense_layers(params)
    assert [w.shape for w, _ in layers] == [(33, 12), (12, 12), (12, 1)] and width == 1.0
    flat = f.pack(params)
    Hp = 16
    assert flat.size == 33 * Hp + Hp + (Hp * Hp + Hp) + Hp + 4
    w1 = flat[:33 * Hp].reshape(33, Hp)
    np.testing.assert_array_equal(w1[:, :12], layers[0][0])
    assert not w1[:, 12:].any()
    assert flat[-4] == np.float32(layers[-1][1][0]) and flat[-3] == 1.0
    init_l, xc_l = _build("local", g)
    pl = init_l(3)
    fl = xc_l.functional
    assert fl.local and fl.negativity and not fl.self_interaction and fl.width_padded == 64
    assert [w.shape for w, _ in fl.dense_layers(pl)[0]] == [(1, 64), (64, 64), (64, 64), (64, 1)]


def test_interface_checks():
    from qex_gb300 import networks

    g = _grids(33)
    with pytest.raises(ValueError):
        networks.LocalMLP({"use_amplitude_encoding": True})
    with pytest.raises(ValueError):
        networks.GlobalMLP({"use_amplitude_encoding": False})
    with pytest.raises(ValueError):  # a within-layer normalisation: not on the GPU path
        _build("local", g, activation="softmax")
    with pytest.raises(ValueError):  # local network under a global network type
        networks.build_xc_functional(networks.LocalMLP().build_network(g), g,
                                     {"network_type": "mlp_ksr"})
    with pytest.raises(ValueError):
        networks.LocalMLP().build_network(None)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def qx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qex_gb300
    from qex_gb300 import od

    return qex_gb300, od


CASES = [
    ("local", {}, "local"),
    ("local", {}, "amplitude"),
    ("local", {"wrap_self_interaction": True, "activation": "gelu", "n_neurons": 20}, "local"),
    ("global", {}, "amplitude"),
    ("global", {"wrap_with_negative_transform": False, "activation": "softplus",
                "n_layers": 2}, "amplitude"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,cfg,convention", CASES)
def test_eval_matches_oracle(qx, kind, cfg, convention):
    qex, od = qx
    from qex_gb300.od.xc_eval import xc_energy_and_potential

    g = _grids(129)
    init_fn, xc_fn = _build(kind, g, **cfg)
    params = init_fn(7)
    oxc = _oracle_xc(xc_fn.functional, params, g, np.float64)
    for r in (0.5, 1.3):
        n = _density(g, r)
        e, v, f = xc_energy_and_potential(n, qex.Partial(xc_fn, params=params), g, convention)
        e_r = o.xc_energy(n, oxc, g, convention)
        v_r = o.xc_potential(n, oxc, g, convention)
        assert abs(e - e_r) <= 2e-6 * max(abs(e_r), 1e-3), (e, e_r)
        np.testing.assert_allclose(f, oxc.values(n), rtol=0, atol=2e-6 * np.abs(oxc.values(n)).max())
        np.testing.assert_allclose(v, v_r, rtol=0, atol=1e-5 * np.abs(v_r).max())


@pytest.mark.gpu
@pytest.mark.parametrize("kind,cfg,convention", CASES)
def test_scf_matches_oracle(qx, kind, cfg, convention):
    """GlobalMLP through kohn_sham_amplitude_encoded (the scan driver), LocalMLP
    through jax_dft kohn_sham (local convention) and the amplitude scan, against
    the oracle's SCF with the same FP32 network arithmetic."""
    qex, od = qx
    g = _grids(129)
    init_fn, xc_fn = _build(kind, g, **cfg)
    params = init_fn(11)
    xc = qex.Partial(xc_fn, params=params)
    oxc = _oracle_xc(xc_fn.functional, params, g, np.float32)
    r, z, ne, T = [-0.7, 0.7], [1.0, 1.0], 2, 8
    ve = o.get_atomic_chain_potential(g, r, z, o.exponential_coulomb)
    n0, _, _ = o.solve_noninteracting_system(ve, ne, g, 5, "banded")
    if convention == "amplitude":
        st = od.jit_scf.kohn_sham_amplitude_encoded(r, z, ne, T, g, xc,
                                                    od.utils.exponential_coulomb, n0,
                                                    num_mixing_iterations=1)
    else:
        st = od.jit_scf.kohn_sham(r, z, ne, T, g, xc, od.utils.exponential_coulomb, n0,
                                  num_mixing_iterations=1)
    ref = o.kohn_sham(r, z, ne, T, g, oxc, o.exponential_coulomb, n0, num_mixing_iterations=1,
                      convention=convention, method="banded")
    np.testing.assert_allclose(st.total_energy, ref["total_energy"], atol=2e-6, rtol=0)
    for a, b in zip(st.density, ref["density"]):
        assert np.sqrt(np.sum((a - b) ** 2) * 0.08) < 1e-6
    assert np.isfinite(st.total_energy).all()


@pytest.mark.gpu
def test_ragged_local_batch_and_global_grid_check(qx):
    """A ragged batch with LocalMLP: each molecule alone equals it in the batch
    (bitwise); a global network refuses molecules whose grid is not its input size."""
    qex, od = qx
    init_fn, xc_fn = _build("local", _grids(129))
    params = init_fn(5)
    xc = qex.Partial(xc_fn, params=params)
    mols = [od.Molecule1D(num_grids=n, grid_spacing=0.08, locations=[-0.8, 0.9],
                          nuclear_charges=[1.0, 1.0], num_electrons=2) for n in (129, 97, 161)]
    cfg = od.SolveConfig(num_iterations=6, convention="local", stencil=5)
    eng = od.engine.default_engine()
    out = eng.solve(od.PackedBatch(mols), xc, cfg)
    e_all = out["energy"].cpu().numpy()
    for i, m in enumerate(mols):
        alone = eng.solve(od.PackedBatch([m]), xc, cfg)["energy"].cpu().numpy()[0]
        np.testing.assert_array_equal(alone, e_all[i])
    g = _grids(129)
    init_g, xc_g = _build("global", g)
    pg = init_g(1)
    cfg_a = od.SolveConfig(num_iterations=3, convention="amplitude", stencil=5)
    out = eng.solve(od.PackedBatch(mols), qex.Partial(xc_g, params=pg), cfg_a)
    st = out["status"].cpu().numpy()
    assert st[0] == 0 and st[1] == 1 and st[2] == 1  # QEX_BAD_ARG beside a good molecule
