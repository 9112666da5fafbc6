"""The multi-GPU path of bench.py is replicas only: each rank runs the whole search
and the ranks meet on the host.  Two gloo ranks on CPU check the combination (the
slowest rank's time, the sum of verified roots)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, v = bench.combine_ranks(100.0 + 50.0 * rank, 3 + rank, world)
    q.put((rank, ms, v))
    dist.destroy_process_group()


def test_two_gloo_replicas_combine():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    for _, ms, v in res:
        assert ms == 150.0 and v == 7.0


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(12.5, 4, 1) == (12.5, 4.0)
