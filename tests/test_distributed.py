"""Replicas across ranks, checked with two gloo processes on the CPU.

Every replica lands on exactly one rank, in whole chi ladders, and the scalar
reductions the benchmark uses (max of the per-rank time, sum of the per-rank
move counts) give the whole-job figures."""
import os
import socket

import pytest

from chromo_gb300.distributed import shard


def test_shard_covers_every_replica_once_in_whole_ladders():
    for n, ladder in ((256, 16), (32, 8), (48, 16), (7, 1)):
        for world in (1, 2, 3, 4, 8):
            got = [list(shard(n, r, world, ladder)) for r in range(world)]
            flat = [i for g in got for i in g]
            assert flat == list(range(n))
            for g in got:
                assert len(g) % ladder == 0
            sizes = [len(g) for g in got]
            assert max(sizes) - min(sizes) <= ladder
    with pytest.raises(ValueError):
        shard(30, 0, 2, 16)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from chromo_gb300 import distributed
    r, w, _ = distributed.init("gloo")
    mine = shard(256, r, w, 16)
    total = distributed.allreduce(len(mine), "sum", w, "gloo")
    slowest = distributed.allreduce(10.0 + r, "max", w, "gloo")
    distributed.barrier(w)
    out.put((r, mine.start, mine.stop, total, slowest))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_replicas_and_reduce():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(a, b) for _, a, b, _, _ in res] == [(0, 128), (128, 256)]
    assert all(t == 256.0 and m == 11.0 for *_, t, m in res)
