"""Multi-GPU mode is replicas only (independent solves per GPU, no data-path
collective); the bench's max-over-ranks aggregation is checked with two gloo
ranks on CPU."""

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
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    value, t = bench.replica_aggregate(1.0 + rank, 100.0, world)
    q.put((rank, value, t))
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t in out:
        assert t == 2.0  # max over ranks
        assert value == 2 * 100.0 / 2.0  # world * units / max time


def test_replica_aggregate_single():
    import bench

    assert bench.replica_aggregate(0.5, 10.0, 1) == (20.0, 0.5)
