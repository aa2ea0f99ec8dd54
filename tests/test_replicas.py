"""Multi-process host logic (gloo, world size 2, CPU): sharding of an ensemble
and the max-over-ranks timing / sum-over-ranks units reduction bench.py uses."""
import os
import socket

import pytest

from rheocell_gb300.replicas import shard


def test_shard_partitions():
    items = list(range(64))
    for world in (1, 2, 3, 5, 8):
        parts = [shard(items, r, world) for r in range(world)]
        assert sum(parts, []) == items
        assert max(map(len, parts)) - min(map(len, parts)) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from rheocell_gb300.replicas import reduce_timing
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, units = reduce_timing(10.0 + rank, 100.0 * (rank + 1))
    out[rank] = (ms, units)
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_timing_gloo_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == (11.0, 300.0)
