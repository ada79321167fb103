"""One database partitioned by shard over several device contexts
(inspire/multi_gpu.py), here two partitions on the one GPU of the test box
(their kernels are independent): every served response equals the response
of one context holding the whole database, and the oracle's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(9, 41))


def test_sharded_database_served_equals_single(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire
    from inspire.multi_gpu import MultiGpuServer, ShardedDatabase

    O = oracle_mod
    ctx = O.Ctx()
    rng = np.random.default_rng(12)
    n_entries = 5 * N + 321
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    params = inspire.InspireParams(p=1 << 16)
    sdb = ShardedDatabase(params, W_SEED, 16, db, ENTRY, devices=[0, 0])
    assert sdb.num_shards == 6 and [d.num_shards for d in sdb.dbs] == [3, 3]
    ms = MultiGpuServer(sdb, max_batch=16, max_inflight=2, capacity=64)
    crs1 = inspire.ServerCrs(params, W_SEED, 16, mode="crt_fixed")
    whole = inspire.EncodedDatabase(crs1, db, ENTRY)
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    clients = [O.Client(ctx, seed=s, rng_seed=120 + s) for s in range(2)]
    keys = [c.packing_keys(pack)[0] for c in clients]
    gids = [ms.register_client(inspire.ClientPackingKeys(y_body=k)) for k in keys]
    ids1 = [crs1.register_client(inspire.ClientPackingKeys(y_body=k)) for k in keys]
    idxs = [int(v) for v in rng.integers(0, n_entries, size=24)] + [0, 3 * N - 1, 3 * N, n_entries - 1]
    seeds = np.zeros((len(idxs), 6, 32), np.uint8)
    brows = np.zeros((len(idxs), 6, 2 * N), np.uint64)
    cl = [k % 2 for k in range(len(idxs))]
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = clients[cl[k]].query_seeded(ix % N)
    sids = [ix // N for ix in idxs]
    tickets = ms.submit(sids, seeds, brows, [gids[c] for c in cl])
    assert set(tickets["part"]) == {0, 1}
    got = ms.poll_batch(tickets)
    want = inspire.respond_seeded_batch(crs1, whole, sids, seeds, brows, [ids1[c] for c in cl])
    assert np.array_equal(got, want)
    for k, ix in enumerate(idxs):
        assert np.array_equal(clients[cl[k]].extract_inspiring(got[k], ENTRY), db[ix * ENTRY:(ix + 1) * ENTRY])
    k = 3
    one = ctx.respond_inspiring(ctx.encode_shard(db, ENTRY, sids[k]), ctx.expand_rgsw(seeds[k], brows[k]), W_SEED,
                                mode=O.MODE_CRT_FIXED, pack=pack, y_body=keys[cl[k]])
    assert np.array_equal(got[k], one)
    ms.close()
    sdb.close()
    whole.close()
    crs1.close()
