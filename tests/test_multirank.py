"""Multi-rank host logic on CPU (gloo, world size 2): shard routing covers
every shard exactly once, batches split by owner, and throughput aggregates as
sum(units) / max(seconds), as bench.py does across GPUs."""
import os

import pytest


def test_router_partitions_every_shard_once():
    from inspire.routing import ShardRouter

    r = ShardRouter(2048, 8192, 3)
    owners = [r.owner(s) for s in range(8192)]
    assert sorted(set(owners)) == [0, 1, 2]
    seen = {(r.owner(s), r.local_shard(s)) for s in range(8192)}
    assert len(seen) == 8192
    assert r.route(2048 * 5000 + 7) == (r.owner(5000), r.local_shard(5000), 7)
    with pytest.raises(KeyError, match="Shard 8192 not found"):
        r.owner(8192)
    parts = r.split([0, 8191, 2731, 5462])
    assert sum(len(v) for v in parts.values()) == 4


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from inspire.routing import ShardRouter, aggregate_throughput

    r = ShardRouter(2048, 1000, world)
    mine = [s for s in range(1000) if r.owner(s) == rank]
    # each rank "answers" its shards; rank 1 is slower
    v = aggregate_throughput(units=len(mine), seconds=1.0 + rank)
    q.put((rank, len(mine), v))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_aggregate():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res[0][1] + res[1][1] == 1000
    assert res[0][2] == res[1][2] == pytest.approx(1000 / 2.0)
