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


def test_multi_gpu_server_routes_and_reassembles():
    """MultiGpuServer's host logic without a GPU: queries split by owning
    partition with local shard ids and per-partition client ids, tickets
    collected back in the caller's order; unknown shards refused."""
    from types import SimpleNamespace

    import numpy as np

    from inspire.multi_gpu import MultiGpuServer
    from inspire.params import InspireParams
    from inspire.routing import ShardRouter

    class FakeCrs:
        def __init__(self, base):
            self.base, self.n = base, 0

        def register_client(self, keys):
            self.n += 1
            return self.base + self.n

        def release_client(self, cid):
            pass

    class FakeServer:
        def __init__(self, part):
            self.part, self.q, self.n = part, {}, 0

        def submit(self, db, local, seeds, b_rows, cids):
            t = np.arange(self.n, self.n + len(local), dtype=np.uint64)
            for k in range(len(local)):
                self.q[int(t[k])] = (self.part, int(local[k]), int(cids[k]), int(seeds[k, 0, 0]))
            self.n += len(local)
            return t, 0

        def poll_batch(self, tickets, out, timeout_us):
            for i, t in enumerate(tickets):
                out[i, 0, :4] = self.q.pop(int(t))
            return np.zeros(len(tickets))

    router = ShardRouter(2048, 10, 3)  # 4 + 4 + 2 shards
    sdb = SimpleNamespace(router=router, dbs=[None] * 3, crs=[FakeCrs(100 * p) for p in range(3)],
                          params=InspireParams())
    ms = MultiGpuServer(sdb, servers=[FakeServer(p) for p in range(3)])
    c0, c1 = ms.register_client(None), ms.register_client(None)
    shards = [9, 0, 4, 3, 8, 5, 1]
    seeds = np.zeros((7, 6, 32), np.uint8)
    seeds[:, 0, 0] = np.arange(7)
    tickets = ms.submit(shards, seeds, np.zeros((7, 6, 4096), np.uint64), [c0, c1, c0, c1, c0, c1, c0])
    out = ms.poll_batch(tickets)
    for k, s in enumerate(shards):
        part, local = router.owner(s), router.local_shard(s)
        cid = (100 * part) + (1 if k % 2 == 0 else 2)
        assert list(out[k, 0, :4]) == [part, local, cid, k]
    with pytest.raises(KeyError, match="Shard 10 not found"):
        ms.submit([10], seeds[:1], np.zeros((1, 6, 4096), np.uint64), [c0])
