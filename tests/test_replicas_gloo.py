"""The multi-GPU form is replicas only: each rank solves its own batch and the
job's throughput combines the ranks (slowest step time, summed work).  This
host logic runs here as two gloo ranks on CPU."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r: step 0.05 + 0.01 r s, e2e 0.06 + 0.01 r s, 10 + r converged of 100
    res = bench.combine_ranks(0.05 + 0.01 * rank, 0.06 + 0.01 * rank, 10 + rank, 100, world, "cpu")
    out.put((rank, res))
    dist.destroy_process_group()


def test_two_replicas_combine_as_max_time_and_summed_work():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        step_s, e2e_s, conv, total = results[r]
        assert abs(step_s - 0.06) < 1e-12 and abs(e2e_s - 0.07) < 1e-12
        assert conv == 21 and total == 200
