"""GPU test of qex_ks1d_solve_static, the entry point that allocates nothing.

Callers that cannot call cudaMalloc at solve time (code inside another
framework's memory pool, or a runtime that forbids allocation on its hot path)
use qex_ks1d_solve_static, whose scratch is a fixed 16 MiB device array in the
library.  This test calls it through the C ABI twice in a row and checks both
results against qex_ks1d_solve with a caller-provided workspace, to the FP64
parity tolerances of the other tests (energies 1e-8 Ha, density L2 1e-7).  It
also checks that a batch too large for the fixed scratch is refused with
QEX_OOM before anything runs.  The file sorts last so that a run stopping at
its first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qex_gb300
    from qex_gb300 import _native as N
    from qex_gb300.od import engine as eng, workloads

    lib = N.load()
    lib.qex_ks1d_solve_static.restype = ctypes.c_int
    lib.qex_ks1d_solve_static.argtypes = [ctypes.POINTER(N.Ks1dBatch),
                                          ctypes.POINTER(N.Ks1dOptions),
                                          ctypes.POINTER(N.XcSpec),
                                          ctypes.POINTER(N.Ks1dOutputs), ctypes.c_void_p]
    return torch, qex_gb300, N, eng, workloads, lib


def test_static_scratch_solve_matches_workspace_solve():
    torch, qex, N, eng, workloads, lib = _setup()
    mols = workloads.batched_molecules(12, seed=21)
    batch = eng.PackedBatch(mols, sort=False)
    cfg = eng.SolveConfig(num_iterations=10, convention="local", stencil=5)
    engine = eng.Ks1dEngine()
    records = ("energy", "final_density")
    ref = engine.solve(batch, qex.LDAExpCoulomb(), cfg, records=records, bucketed=False)
    ref_e = ref["energy"].cpu().numpy()
    ref_d = ref["final_density"].cpu().numpy()

    opts = eng._options(cfg, batch, False)
    spec, keep = qex.LDAExpCoulomb().spec(None, N.QEX_XC_LOCAL)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        out = engine.allocate_outputs(batch, cfg, records)
        cb = batch.c_batch()
        co = engine._c_outputs(out)
        rc = lib.qex_ks1d_solve_static(ctypes.byref(cb), ctypes.byref(opts), ctypes.byref(spec),
                                       ctypes.byref(co), stream)
        assert rc == N.QEX_OK, (call, rc)
        torch.cuda.synchronize()
        e = out["energy"].cpu().numpy()
        d = out["final_density"].cpu().numpy()
        np.testing.assert_allclose(e, ref_e, atol=1e-8, rtol=0)
        for a, b in zip(batch.split(d), batch.split(ref_d)):
            assert float(np.sqrt(np.sum((a - b) ** 2) * 0.08)) < 1e-7


def test_static_scratch_rejects_oversized_batch():
    torch, qex, N, eng, workloads, lib = _setup()
    mols = workloads.batched_molecules(512, seed=3)
    batch = eng.PackedBatch(mols, sort=False)
    cfg = eng.SolveConfig(num_iterations=10, convention="local", stencil=5)
    opts = eng._options(cfg, batch, False)
    need = ctypes.c_size_t()
    assert lib.qex_ks1d_workspace_size(ctypes.byref(opts), batch.size, ctypes.byref(need)) == 0
    assert need.value > (16 << 20)
    engine = eng.Ks1dEngine()
    out = engine.allocate_outputs(batch, cfg, ("energy",))
    spec, keep = qex.LDAExpCoulomb().spec(None, N.QEX_XC_LOCAL)
    cb = batch.c_batch()
    co = engine._c_outputs(out)
    rc = lib.qex_ks1d_solve_static(ctypes.byref(cb), ctypes.byref(opts), ctypes.byref(spec),
                                   ctypes.byref(co),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.QEX_OOM
