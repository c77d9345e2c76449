"""The multi-rank path of bench.py (N replicas, one per GPU) on CPU with the
gloo backend, world size 2: the reported time is the slowest rank's and the
throughput counts every rank's particles."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, value = bench.aggregate_ranks(10.0 * (rank + 1), 1000 * (rank + 1), 5, dist)
    dist.barrier()
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in res:
        assert ms == 20.0                     # max over ranks
        assert abs(value - 3000 * 5 / 0.020) < 1e-6  # all ranks' particles
