"""The N > 1 bench path on the CPU: registrations are independent, so N ranks run N
replicas and the whole-job rate is the units of all ranks over the slowest rank's
time (bench.replica_rate, a MAX all-reduce).  Two gloo ranks with different times
must both report 2 x units / max time."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rate, ms = bench.replica_rate(12, 1000.0 * (rank + 1), dist, "cpu")
        with open(os.path.join(out_dir, "r%d.json" % rank), "w") as fh:
            json.dump({"rate": rate, "ms": ms}, fh)
    finally:
        dist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        d = json.load(open(tmp_path / ("r%d.json" % r)))
        assert d["ms"] == 2000.0
        assert d["rate"] == pytest.approx(12 * world / 2.0)


def test_replica_rate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    rate, ms = bench.replica_rate(8, 500.0)
    assert ms == 500.0 and rate == pytest.approx(16.0)
