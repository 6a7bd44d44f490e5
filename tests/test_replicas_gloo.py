"""CPU: the bench's multi-GPU path is data-parallel replicas (each rank runs
its own batch, no collective on the data path); its only collective is the
max-over-ranks of the step times.  Exercised with world_size 2 on gloo."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # rank r took 10 (r + 1) ms per step and 20 (r + 1) ms end to end
    ms, rate = bench.aggregate_replicas([10.0 * (rank + 1), 20.0 * (rank + 1)], 64, world, torch.device("cpu"))
    q.put((rank, ms, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in out:
        assert ms == [20.0, 40.0]                      # max over ranks
        assert rate == pytest.approx([2 * 64 / 0.020, 2 * 64 / 0.040])  # all ranks' circuits


def test_replica_aggregation_single_process():
    import bench

    ms, rate = bench.aggregate_replicas([25.0], 64, 1, torch.device("cpu"))
    assert ms == [25.0] and rate == pytest.approx([2560.0])
