"""The benchmark configurations' own shapes, bit-exact against the oracle:
C1 (the crate's CPU-runnable case: 1024 entries x 32 B, InsPIRe^1 with a
full query and InsPIRe^2 with a seeded one, index uniform in [0, 1024)) and
a C4 batch whose queries all hit one shard."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(50, 82))


@pytest.fixture(scope="module")
def c1(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    db = np.random.default_rng(1).integers(0, 256, size=1024 * ENTRY, dtype=np.uint8)
    ctx = O.Ctx()
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    client = O.Client(ctx, seed=0, rng_seed=3)
    shard = ctx.encode_shard(db, ENTRY, 0)
    return dict(O=O, inspire=inspire, ctx=ctx, crs=crs, edb=edb, pack=pack, client=client, shard=shard, db=db)


def test_c1_inspire1_and_inspire2(c1):
    W = c1
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    assert W["edb"].num_shards == 1
    y_body, _ = client.packing_keys(W["pack"])
    keys = inspire.ClientPackingKeys(y_body=y_body)
    for idx in np.random.default_rng(2).integers(0, 1024, size=4):
        idx = int(idx)
        seeds, b_rows = client.query_seeded(idx)
        rgsw = ctx.expand_rgsw(seeds, b_rows)
        want = ctx.respond_inspiring(W["shard"], rgsw, W_SEED, mode=W["O"].MODE_CRT_FIXED, pack=W["pack"],
                                     y_body=y_body)
        full = inspire.respond_inspiring(W["crs"], W["edb"], inspire.ClientQuery(0, rgsw, inspiring_packing_keys=keys))
        seeded = inspire.respond_seeded_inspiring(W["crs"], W["edb"],
                                                  inspire.SeededClientQuery(0, seeds, b_rows, inspiring_packing_keys=keys))
        for r in (full, seeded):
            assert np.array_equal(np.stack([r.ciphertext.a, r.ciphertext.b]), want)
        assert np.array_equal(client.extract_inspiring(want, ENTRY), W["db"][idx * ENTRY:(idx + 1) * ENTRY])
    # coefficients beyond the 1024 entries are zero: an index past them reads zeros
    seeds, b_rows = client.query_seeded(1500)
    r = inspire.respond_seeded_inspiring(W["crs"], W["edb"],
                                         inspire.SeededClientQuery(0, seeds, b_rows, inspiring_packing_keys=keys))
    got = client.extract_inspiring(np.stack([r.ciphertext.a, r.ciphertext.b]), ENTRY)
    assert not got.any()


def test_c4_same_shard_batch(c1):
    """B queries against one shard in one launch (the shard's contracted form
    is shared through L2): each response equals the single-query one."""
    W = c1
    inspire, client = W["inspire"], W["client"]
    y_body, _ = client.packing_keys(W["pack"])
    cid = W["crs"].register_client(inspire.ClientPackingKeys(y_body=y_body))
    idxs = list(np.random.default_rng(4).integers(0, 1024, size=32))
    seeds = np.zeros((32, 6, 32), np.uint8)
    brows = np.zeros((32, 6, 2 * N), np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = client.query_seeded(int(ix))
    out = inspire.respond_seeded_batch(W["crs"], W["edb"], [0] * 32, seeds, brows, [cid] * 32)
    for k in (0, 7, 31):
        one = inspire.respond_seeded_batch(W["crs"], W["edb"], [0], seeds[k:k + 1], brows[k:k + 1], [cid])[0]
        assert np.array_equal(out[k], one)
        ix = int(idxs[k])
        assert np.array_equal(client.extract_inspiring(out[k], ENTRY), W["db"][ix * ENTRY:(ix + 1) * ENTRY])
    W["crs"].release_client(cid)
