"""GPU tests of the continuous-batching server: every served result equals the
same request solved alone (the kernel is deterministic per molecule), all
requests complete, and latency statistics are produced."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def srv():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qex_gb300
    from qex_gb300 import serving
    from qex_gb300.od import engine as eng

    cfg = eng.SolveConfig(num_iterations=20, convention="local", stencil=3, alpha=0.5,
                          alpha_decay=0.9, num_mixing_iterations=1)
    return qex_gb300, serving, eng, cfg


def test_served_results_equal_alone(srv):
    qex, serving, eng, cfg = srv
    arrivals = serving.poisson_arrivals(400.0, 0.15, seed=3)
    reqs = serving.config1_requests(arrivals, seed=3)
    # a few requests of other shapes in the mix
    for k, r in enumerate(reqs[::5]):
        r.molecule = eng.Molecule1D(num_grids=257 + 64 * (k % 3), grid_spacing=0.08,
                                    locations=[-1.0, 0.4], nuclear_charges=[2.0, 1.0],
                                    num_electrons=3)
    server = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=4, max_batch=16)
    done = server.serve(reqs)
    assert all(np.isfinite(r.latency) for r in done)
    assert server.launches >= 2  # requests were admitted in more than one batch
    engine = eng.Ks1dEngine()
    for r in done[:: max(1, len(done) // 8)]:
        alone = engine.solve(eng.PackedBatch([r.molecule]), qex.LDAExpCoulomb(), cfg,
                             records=("energy", "final_density"))
        np.testing.assert_array_equal(alone["energy"].cpu().numpy()[0], r.energies)
        np.testing.assert_array_equal(alone["final_density"].cpu().numpy(), r.density)
    s = serving.latency_summary(done)
    assert s["requests"] == len(reqs) and s["p99_ms"] >= s["p50_ms"] > 0


def test_memory_admission_splits_batches(srv):
    qex, serving, eng, cfg = srv
    reqs = serving.config1_requests(np.zeros(12), seed=1)
    one = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=4, max_batch=64)
    est = one._estimate(reqs[:3])
    # a budget that fits about three requests at a time forces several launches
    small = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=4, max_batch=64,
                              memory_budget_bytes=est)
    done = small.serve(reqs, realtime=False)
    assert small.launches >= 4
    assert all(r.energies is not None for r in done)


def test_plain_form_matches_served(srv):
    qex, serving, eng, cfg = srv
    reqs = serving.config1_requests(np.linspace(0, 0.01, 4), seed=5)
    plain = serving.serve_plain(qex.LDAExpCoulomb(), cfg,
                                [serving.Request(r.rid, r.molecule, r.arrival) for r in reqs])
    served = serving.ScfServer(qex.LDAExpCoulomb(), cfg).serve(reqs)
    for a, b in zip(plain, served):
        np.testing.assert_array_equal(a.energies, b.energies)


def test_mixed_1d_3d_stream_equals_alone(srv):
    # config-5 shape: 1D requests batched, 3D requests replaying their resident
    # molecule's captured SCF graph; every result equals the request solved alone
    qex, serving, eng, cfg = srv
    from qex_gb300.td import graph, scf, workloads

    mols3 = {"a": workloads.synthetic_molecule(2, seed=0),
             "b": workloads.synthetic_molecule(3, seed=1)}
    graphs = {k: graph.CapturedScf(m, max_cycle=12) for k, m in mols3.items()}
    reqs = serving.mixed_requests(serving.poisson_arrivals(300.0, 0.1, seed=7), list(mols3),
                                  frac3d=0.3, seed=7)
    server = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=4, max_batch=16,
                               graphs3d=graphs)
    done = server.serve(reqs, realtime=False)
    three = [r for r in done if r.is3d]
    one = [r for r in done if not r.is3d]
    assert three and one
    alone = {k: scf.run_scf(m, max_cycle=12) for k, m in mols3.items()}
    for r in three:
        np.testing.assert_array_equal(r.energies, alone[r.graph3d].energies.cpu().numpy())
        assert r.status == 0
    engine = eng.Ks1dEngine()
    for r in one[:4]:
        a = engine.solve(eng.PackedBatch([r.molecule]), qex.LDAExpCoulomb(), cfg,
                         records=("energy", "final_density"))
        np.testing.assert_array_equal(a["energy"].cpu().numpy()[0], r.energies)
    s = serving.latency_summary(done)
    assert s["3d"]["requests"] == len(three) and s["1d"]["requests"] == len(one)
    # the plain one-at-a-time form gives the same 3D energies (no graph)
    plain = serving.serve_plain(qex.LDAExpCoulomb(), cfg,
                                [serving.Request(r.rid, None, r.arrival, graph3d=r.graph3d)
                                 for r in three[:2]], molecules3d=mols3, max_cycle=12)
    for a, b in zip(plain, three[:2]):
        np.testing.assert_array_equal(a.energies, b.energies)


def test_new_3d_molecules_built_on_admission(srv):
    """3D requests for molecules that are not resident are admitted by building
    them (GPU integrals, then the captured graph) inside the request; the
    result equals the molecule solved alone; admission by free HBM."""
    qex, serving, eng, cfg = srv
    from qex_gb300.td import scf, workloads

    keys = [(2, 21), (3, 22)]
    built = {}

    def build(key):
        built[key] = workloads.device_molecule(key[0], seed=key[1])[0]
        return built[key]

    reqs = serving.mixed_requests(serving.poisson_arrivals(200.0, 0.1, seed=9), keys,
                                  frac3d=0.4, seed=9)
    server = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=4, max_batch=16,
                               builder3d=build)
    done = server.serve(reqs, realtime=False)
    three = [r for r in done if r.is3d]
    assert three and server.built3d == len({r.graph3d for r in three})
    for r in three:
        alone = scf.run_scf(built[r.graph3d], max_cycle=30)
        np.testing.assert_array_equal(r.energies, alone.energies.cpu().numpy())
        assert r.e_tot == float(alone.e_tot.cpu()[0])
        assert r.converged3d == bool(alone.converged.cpu()[0])


def test_deadline_reports_unserved_requests(srv):
    """An overloaded stream cut at its deadline: work in flight completes, the
    requests still waiting come back unserved and the summary counts them."""
    qex, serving, eng, cfg = srv
    reqs = serving.config1_requests(np.zeros(64), seed=2)
    server = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=1, max_batch=4)
    done = server.serve(reqs, realtime=False, deadline=0.0)
    served = [r for r in done if np.isfinite(r.finish)]
    assert len(served) <= 4 and len(served) + sum(1 for r in done if r.energies is None) == 64
    s = serving.latency_summary(done)
    assert s["unserved"] == 64 - len(served)


def test_3d_backlog_does_not_hold_back_1d(srv):
    """The streams split into a 1D and a 3D share: with a backlog of replays of
    one 3D molecule (they run one at a time), the 1D requests that arrive
    beside it are all served long before the backlog drains."""
    qex, serving, eng, cfg = srv
    from qex_gb300.td import graph, workloads

    graphs = {"a": graph.CapturedScf(workloads.synthetic_molecule(3, seed=4), max_cycle=12)}
    three = [serving.Request(i, None, 0.0, graph3d="a") for i in range(40)]
    one = serving.config1_requests(np.zeros(32), seed=5)
    for i, r in enumerate(one):
        r.rid = 100 + i
    server = serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=4, max_batch=16,
                               graphs3d=graphs)
    assert server.max_inflight3d == 2
    done = server.serve(three + one, realtime=False)
    fin1 = max(r.finish for r in done if not r.is3d)
    fin3 = sorted(r.finish for r in done if r.is3d)
    assert fin1 < fin3[len(fin3) // 2], (fin1, fin3[len(fin3) // 2])
    with pytest.raises(ValueError):
        serving.ScfServer(qex.LDAExpCoulomb(), cfg, max_inflight=2, graphs3d=graphs,
                          max_inflight3d=2)
