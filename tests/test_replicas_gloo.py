"""The N-GPU path of the benchmark is N independent replicas (the cycle has
no exchange between GPUs).  Its only cross-rank logic -- job time = slowest
rank, work = sum over ranks -- is checked here with two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units = bench.aggregate(100.0 + 50.0 * rank, 1000 * (rank + 1), world)
    dist.destroy_process_group()
    q.put((rank, ms, units))


def test_replica_aggregation_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, units in res:
        assert ms == 150.0          # the slowest rank
        assert units == 3000        # all ranks' analyses


def test_single_process_aggregation_is_identity():
    import bench
    assert bench.aggregate(12.5, 77, 1) == (12.5, 77)
