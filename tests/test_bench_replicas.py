"""bench.py's N > 1 path on CPU: two gloo ranks, each a replica with its own
device time; the whole-job value uses the slowest rank's time and every
rank's atoms (replicas, weak scaling, no data-path collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dev_ms = [120.0, 150.0][rank]
    value, max_ms = bench.replica_throughput(dev_ms, atoms=1000, steps=10, dist=dist, device="cpu")
    out[rank] = (value, max_ms)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        value, max_ms = out[r]
        assert max_ms == 150.0
        assert value == pytest.approx(2 * 1000 * 10 / 0.150)


def test_replica_throughput_single():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    value, ms = bench.replica_throughput(100.0, atoms=500, steps=4)
    assert ms == 100.0 and value == pytest.approx(500 * 4 / 0.1)
