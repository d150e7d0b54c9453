"""Multi-replica timing of ``bench.py`` on CPU: two ``gloo`` ranks, the job
rate uses the slowest rank's time (max over ranks, as the bench contract
requires) and counts every rank's steps."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    elapsed = [100.0, 250.0][rank]  # ms: rank 1 is the slower replica
    rate, slowest = bench.replica_rate(elapsed, 10, world, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, rate, slowest))


def test_replica_rate_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import socket
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = mp.Queue()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, rate, slowest in out:
        assert slowest == 250.0
        assert rate == pytest.approx(2 * 10 / 0.25)


def test_replica_rate_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench
    rate, slowest = bench.replica_rate(200.0, 5, 1)
    assert slowest == 200.0 and rate == pytest.approx(25.0)
