"""CPU tests of the serving layer's host logic: the seeded request streams
(Poisson arrivals, the 1D/3D mix) and the latency summary (p50/p99, the
converged count, the 1D/3D split).  The GPU admission and the served-equals-
alone identity are in ``test_serving_gpu.py``."""

import numpy as np

from qex_gb300 import serving


def test_poisson_arrivals_are_seeded_sorted_and_inside_the_window():
    a = serving.poisson_arrivals(500.0, 2.0, seed=3)
    b = serving.poisson_arrivals(500.0, 2.0, seed=3)
    np.testing.assert_array_equal(a, b)
    assert np.all(np.diff(a) >= 0.0) and a[0] >= 0.0 and a[-1] <= 2.0
    # count ~ Poisson(1000): within 5 standard deviations
    assert abs(a.size - 1000) < 5 * np.sqrt(1000)


def test_mixed_requests_fraction_shape_and_reproducibility():
    arr = np.linspace(0.0, 1.0, 4000)
    keys = ["a", "b", "c"]
    reqs = serving.mixed_requests(arr, keys, frac3d=0.2, seed=5)
    again = serving.mixed_requests(arr, keys, frac3d=0.2, seed=5)
    assert [r.graph3d for r in reqs] == [r.graph3d for r in again]
    n3 = sum(r.is3d for r in reqs)
    assert abs(n3 / len(reqs) - 0.2) < 0.03
    assert {r.graph3d for r in reqs if r.is3d} == set(keys)
    for r in reqs:
        if r.is3d:
            assert r.molecule is None
        else:
            m = r.molecule
            assert m.num_grids == 513 and m.num_electrons == 2
            loc = np.asarray(m.locations)
            assert np.isclose(loc[0], -loc[1]) and 0.5 <= loc[1] <= 1.5
    assert [r.rid for r in reqs] == list(range(len(arr)))
    assert all(r.arrival == t for r, t in zip(reqs, arr))
    # no resident 3D molecules: every request is 1D
    assert not any(r.is3d for r in serving.mixed_requests(arr[:50], [], seed=1))


def test_config1_requests_match_the_plain_configuration():
    reqs = serving.config1_requests([0.0, 0.5, 1.0], seed=2)
    for r in reqs:
        m = r.molecule
        assert m.num_grids == 513 and m.grid_spacing == 0.08
        assert list(m.nuclear_charges) == [1.0, 1.0] and m.num_electrons == 2
        assert not r.is3d


def _done(rid, arrival, latency, dE, status=0, graph=None):
    r = serving.Request(rid=rid, molecule=None, arrival=arrival, graph3d=graph)
    r.start = arrival
    r.finish = arrival + latency
    r.energies = np.array([-1.0, -1.0 + dE])
    r.status = status
    if graph is not None:  # a 3D result carries the device's stop-rule flag
        r.converged3d = dE < 1e-8
    return r


def test_latency_summary_percentiles_converged_count_and_split():
    lat = np.linspace(0.001, 0.1, 100)
    reqs = []
    for i, l in enumerate(lat):
        dE = 1e-9 if i % 4 else 1e-6        # every fourth not converged
        status = 0x1 if i == 1 else 0        # a flagged solve does not count
        reqs.append(_done(i, 0.01 * i, l, dE, status, graph="m" if i % 5 == 0 else None))
    s = serving.latency_summary(reqs)
    assert s["requests"] == 100
    assert s["converged"] == 100 - 25 - 1
    np.testing.assert_allclose(s["p50_ms"], np.percentile(lat, 50) * 1e3)
    np.testing.assert_allclose(s["p99_ms"], np.percentile(lat, 99) * 1e3)
    span = max(r.finish for r in reqs) - min(r.arrival for r in reqs)
    np.testing.assert_allclose(s["solves_per_s"], 100 / span)
    assert s["3d"]["requests"] == 20 and s["1d"]["requests"] == 80
    assert s["1d"]["span_s"] == s["span_s"]
    # a per-molecule flag (here the degenerate-frontier bit) also excludes it
    r = _done(0, 0.0, 0.01, 1e-9, status=0x100)
    assert serving.latency_summary([r, _done(1, 0.0, 0.02, 1e-9)])["converged"] == 1


def test_plan_tuner_key_is_the_shape_histogram():
    """The launch-plan cache key: molecules per (grid size, eigenpair count)
    class plus the XC kind and the solve options, independent of order."""
    import dataclasses

    from qex_gb300.od.autotune import PlanTuner
    from qex_gb300.od.engine import SolveConfig

    @dataclasses.dataclass
    class M:
        num_electrons: int

    @dataclasses.dataclass
    class B:
        num_grids_host: list
        molecules: list

    cfg = SolveConfig()
    a = B([513, 257, 513], [M(2), M(3), M(2)])
    b = B([257, 513, 513], [M(3), M(2), M(2)])
    ka, kb = PlanTuner.key(a, 3, cfg), PlanTuner.key(b, 3, cfg)
    assert ka == kb
    assert ka[0] == ((257, 2, 1), (513, 2, 2))
    assert PlanTuner.key(a, 4, cfg) != ka
    assert PlanTuner.key(a, 3, dataclasses.replace(cfg, stencil=3)) != ka
    c = B([513, 257, 513], [M(4), M(3), M(2)])  # one molecule moves to K = 3
    assert PlanTuner.key(c, 3, cfg) != ka


def test_staged_molecule_setup_state_machine():
    """A new 3D molecule's set-up advances one stage per call; the molecule
    becomes resident after the last stage, and a stage that fails leaves no
    half-built molecule behind (host logic only, no GPU)."""
    import pytest

    from qex_gb300.serving import ScfServer

    srv = ScfServer.__new__(ScfServer)
    srv.graphs3d, srv.resident, srv.built3d, srv._building = {}, 0, 0, None

    class Graph:
        nbytes = 10

    done = []

    def stages():
        done.append(1)
        yield
        done.append(2)
        yield
        done.append(3)

    g = Graph()
    srv._building = ("a", g, stages())
    srv._advance_build()
    assert srv._building is not None and done == [1]
    srv._advance_build()
    assert done == [1, 2] and "a" not in srv.graphs3d
    srv._advance_build()
    assert srv._building is None and srv.graphs3d == {"a": g}
    assert srv.resident == 10 and srv.built3d == 1

    def failing():
        yield
        raise RuntimeError("out of device memory")

    srv._building = ("b", Graph(), failing())
    srv._advance_build()
    with pytest.raises(RuntimeError):
        srv._advance_build()
    assert srv._building is None and "b" not in srv.graphs3d and srv.built3d == 1
