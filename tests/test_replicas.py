"""Multi-GPU protocol of bench.py (replicas only): each rank runs the whole workload, the step
time is the max over ranks and the value counts every rank's units.  Exercised with two gloo
ranks on CPU; no GPU and no collective on the data path."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
        worst = bench.max_over_ranks(dist, ms)
        dist.barrier()
        q.put((rank, worst, bench.replica_rate(world, 1.0e9, worst)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, worst, rate in got:
        assert worst == 15.0
        assert rate == pytest.approx(2 * 1.0e9 / 15e-3)


def test_single_process_needs_no_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(None, 7.5) == 7.5
    assert bench.replica_rate(1, 100.0, 1000.0) == pytest.approx(100.0)
