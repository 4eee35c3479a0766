"""The N > 1 path of bench.py: independent replicas whose report is the slowest rank's
time and the summed atom-steps (world_size 2, gloo, CPU)."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    res = bench.replica_report([1.0 + rank, 0.5 * (rank + 1)], [100.0 * (rank + 1), 7.0], dist, "cpu")
    out[rank] = res
    dist.destroy_process_group()


def test_replica_report_two_ranks():
    port = _free_port()
    with tmp.Manager() as m:
        out = m.dict()
        tmp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        assert res[r] == (2.0, 1.0, 300.0, 14.0)


def test_replica_report_single_process():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_report([1.5], [10.0]) == (1.5, 10.0)
