"""The multi-GPU path is replicas only: every rank runs the whole workload and
the job's throughput is world x per-rank units over the slowest rank's time.
Exercised here with two gloo ranks on the CPU (no GPU)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took (r + 1) seconds for 1000 units
    value, sec = bench.aggregate(rank + 1.0, 1000.0, dist, "cpu")
    out.put((rank, value, sec))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # max time is 2 s; the job processed 2 x 1000 units
    for _, value, sec in res:
        assert sec == 2.0 and value == pytest.approx(1000.0)


def test_single_process_aggregation():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    value, sec = bench.aggregate(0.5, 100.0)
    assert value == 200.0 and sec == 0.5
