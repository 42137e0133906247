"""The multi-GPU path of bench.py is replicas only (independent copies of the step, no collective on
the data path): two gloo ranks on the CPU check its host logic — the slowest replica's time is the
job's time, and the whole-job rate counts every replica's units."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, device='cpu')
    out.put((rank, ms, bench.whole_job_rate(1000, 4, world, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_the_slowest_rank():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        port = s.getsockname()[1]
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    # 2 replicas x 1000 units x 4 steps in 15 ms
    assert all(abs(r[2] - 2 * 1000 * 4 / 15e-3) < 1e-6 for r in res)


def test_single_process_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, device='cpu') == 3.5
    assert bench.whole_job_rate(10, 2, 1, 4.0) == pytest.approx(5000.0)
