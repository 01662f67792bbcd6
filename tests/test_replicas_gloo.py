"""The N > 1 path of bench.py: independent replicas, one per rank, aggregated with the
slowest rank's time and the sum of every rank's units.  Two gloo ranks on CPU (no GPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    times = [10.0 + rank, 20.0 - rank, 5.0 * (rank + 1)]
    t, u = bench.replica_aggregate(dist, times, 1000 * (rank + 1))
    out[rank] = (t, u)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        t, u = out[r]
        assert t == [11.0, 20.0, 10.0]   # max over ranks per timing
        assert u == 3000.0               # sum of the ranks' units


def test_replica_aggregate_single_rank_is_identity():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.replica_aggregate(None, [1.0, 2.0], 7) == ([1.0, 2.0], 7)
