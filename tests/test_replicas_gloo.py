"""The N>1 host path on CPU: two ranks over gloo (127.0.0.1).  Ranks run
independent replicas (or shards of independent instances); only the timing
and counts are combined: max of the times, sum of the cell-updates."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from samurai_gb300.replicas import reduce_over_ranks, shard_instances  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, n = reduce_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), world, device="cpu")
        sizes = [4.0 ** (7 + (i % 5)) for i in range(23)]
        mine = shard_instances(sizes, rank, world)
        out.put((rank, ms, n, mine))
    finally:
        dist.destroy_process_group()


def test_two_ranks_reduce_and_shard():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, ms, n, _ in res:
        assert ms == 15.0 and n == 3000.0
    shards = [set(r[3]) for r in res]
    assert shards[0].isdisjoint(shards[1]) and shards[0] | shards[1] == set(range(23))
    sizes = [4.0 ** (7 + (i % 5)) for i in range(23)]
    loads = [sum(sizes[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(sizes)


def test_single_rank_is_identity():
    assert reduce_over_ranks(3.5, 42, 1) == (3.5, 42.0)
    assert shard_instances([1.0, 2.0, 3.0], 0, 1) == [0, 1, 2]
