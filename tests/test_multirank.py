"""Multi-rank host logic on CPU (gloo, world size 2): the bench runs one
replica per GPU and reports the slowest rank's time; every rank must agree on
it. No GPU is involved."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, values, out):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    out[rank] = bench.max_over_ranks(values[rank], world, torch.device("cpu"))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    values = [12.5, 37.25]
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, values, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0] == out[1] == max(values)


def test_max_over_ranks_single():
    import bench

    assert bench.max_over_ranks(3.5, 1, None) == 3.5


def test_dist_info_defaults(monkeypatch):
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_info() == (0, 1, 0)
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.dist_info() == (1, 2, 1)
