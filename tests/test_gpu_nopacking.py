"""GPU parity of the NoPacking Respond path (respond / respond_seeded,
src/pir/respond.rs:71-115 and 408-415) through the C ABI, bit-exact against
the oracle restatement, plus extraction of the entry from the column
ciphertexts (the crate's NoPacking client: decrypt each column, coefficient
0 holds the column value) and the crate's error behaviour."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(3, 35))


@pytest.fixture(scope="module")
def world(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(77)
    n_entries = 2 * N + 300  # three shards, the last one partial
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    ctx = O.Ctx()
    client = O.Client(ctx, seed=5, rng_seed=23)
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    shards = [ctx.encode_shard(db, ENTRY, s) for s in range(3)]
    return dict(O=O, inspire=inspire, ctx=ctx, client=client, db=db, crs=crs, edb=edb, shards=shards)


def entry_from_columns(client, cols):
    """reconstruct_entry (encode_db.rs:186-201) over per-column decryptions."""
    out = np.zeros(ENTRY, dtype=np.uint8)
    for c in range(cols.shape[0]):
        v = int(client.decrypt(cols[c])[0])
        out[2 * c] = v & 0xFF
        out[2 * c + 1] = (v >> 8) & 0xFF
    return out


@pytest.mark.parametrize("index", [0, 1, 2047, 2048, 4096 + 299])
def test_seeded_nopacking_bit_exact(world, index):
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    sid, local = divmod(index, N)
    seeds, b_rows = client.query_seeded(local)
    want, want_cols = ctx.respond_nopacking(W["shards"][sid], ctx.expand_rgsw(seeds, b_rows), with_columns=True)
    resp = inspire.respond_seeded(W["crs"], W["edb"], inspire.SeededClientQuery(sid, seeds, b_rows))
    assert len(resp.column_ciphertexts) == 16
    assert np.array_equal(resp.ciphertext.a, want[0])
    assert np.array_equal(resp.ciphertext.b, want[1])
    got_cols = np.stack([np.stack([c.a, c.b]) for c in resp.column_ciphertexts])
    assert np.array_equal(got_cols, want_cols)
    expect = W["db"][index * ENTRY:(index + 1) * ENTRY]
    assert np.array_equal(entry_from_columns(client, got_cols), expect)


def test_unseeded_nopacking_and_variant(world):
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    seeds, b_rows = client.query_seeded(1500)
    rgsw = ctx.expand_rgsw(seeds, b_rows)
    want, want_cols = ctx.respond_nopacking(W["shards"][1], rgsw, with_columns=True)
    q = inspire.ClientQuery(1, rgsw)
    resp = inspire.respond(W["crs"], W["edb"], q)
    assert np.array_equal(np.stack([resp.ciphertext.a, resp.ciphertext.b]), want)
    assert np.array_equal(np.stack([np.stack([c.a, c.b]) for c in resp.column_ciphertexts]), want_cols)
    # respond_with_variant / respond_seeded_with_variant route NoPacking here
    # whatever the packing keys (respond.rs:135, 167)
    r2 = inspire.respond_with_variant(W["crs"], W["edb"], q, inspire.InspireVariant.NoPacking)
    assert np.array_equal(r2.ciphertext.b, want[1])
    r3 = inspire.respond_seeded_with_variant(W["crs"], W["edb"], inspire.SeededClientQuery(1, seeds, b_rows),
                                             inspire.InspireVariant.NoPacking)
    assert np.array_equal(r3.ciphertext.a, want[0])
    assert len(r3.column_ciphertexts) == 16


@pytest.mark.parametrize("index", [9, 2048 + 777, 4096 + 299])
def test_combined_only_matches(world, index):
    """Without column ciphertexts the kernel transforms the digit sums over
    the columns once (one NTT per digit instead of one per column and digit);
    the combined ciphertext must equal the oracle's sum of the column
    products, and the with-columns path's, bit for bit (full and partial
    shards)."""
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    sid, local = divmod(index, N)
    seeds, b_rows = client.query_seeded(local)
    want = ctx.respond_nopacking(W["shards"][sid], ctx.expand_rgsw(seeds, b_rows))
    q = inspire.SeededClientQuery(sid, seeds, b_rows)
    resp = inspire.respond_seeded(W["crs"], W["edb"], q, with_columns=False)
    assert resp.column_ciphertexts == []
    assert np.array_equal(np.stack([resp.ciphertext.a, resp.ciphertext.b]), want)
    full = inspire.respond_seeded(W["crs"], W["edb"], q)
    assert np.array_equal(full.ciphertext.b, resp.ciphertext.b)
    assert np.array_equal(full.ciphertext.a, resp.ciphertext.a)


def test_nopacking_batch_equals_single(world):
    W = world
    inspire, client = W["inspire"], W["client"]
    idxs = [3, 2049, 4100, 2047]
    seeds = np.zeros((len(idxs), 6, 32), dtype=np.uint8)
    brows = np.zeros((len(idxs), 6, 2 * N), dtype=np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = client.query_seeded(ix % N)
    sids = [ix // N for ix in idxs]
    out = inspire.respond_seeded_nopacking_batch(W["crs"], W["edb"], sids, seeds, brows)
    pinned = inspire.pir.PinnedBuffer(out.shape, np.uint64)
    got = inspire.respond_seeded_nopacking_batch(W["crs"], W["edb"], sids, seeds, brows, out=pinned.array)
    assert got is pinned.array and np.array_equal(got, out)
    pinned.close()
    with pytest.raises(ValueError):
        inspire.respond_seeded_nopacking_batch(W["crs"], W["edb"], sids, seeds, brows, out=np.empty((1, 2, 2 * N)))
    for k in range(len(idxs)):
        r = inspire.respond_seeded(W["crs"], W["edb"], inspire.SeededClientQuery(sids[k], seeds[k], brows[k]),
                                   with_columns=False)
        assert np.array_equal(out[k], np.stack([r.ciphertext.a, r.ciphertext.b]))


def test_nopacking_shard_not_found(world):
    W = world
    inspire, client = W["inspire"], W["client"]
    seeds, b_rows = client.query_seeded(0)
    with pytest.raises(inspire.PirError, match="Shard 3 not found"):
        inspire.respond_seeded(W["crs"], W["edb"], inspire.SeededClientQuery(3, seeds, b_rows))
    with pytest.raises(inspire.PirError, match="Shard 7 not found"):
        inspire.respond_seeded_nopacking_batch(W["crs"], W["edb"], [0, 7], np.zeros((2, 6, 32), np.uint8),
                                               np.zeros((2, 6, 2 * N), np.uint64))


@pytest.mark.parametrize("entry_size,gamma", [(2, 1), (4, 2), (16, 8)])
def test_nopacking_other_column_counts(oracle_mod, entry_size, gamma):
    """NoPacking with fewer columns (gamma = 1, 2, 8), full and partial
    shards: the combined-only path (digit sums) and the with-columns path (a
    single query: its columns split over CTAs), against the oracle.  Column
    counts that are not powers of two are refused by the GPU path."""
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(100 + entry_size)
    n_entries = N + 500
    db = rng.integers(0, 256, size=n_entries * entry_size, dtype=np.uint8)
    ctx = O.Ctx()
    client = O.Client(ctx, seed=2, rng_seed=entry_size)
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, gamma, mode="crt_fixed")
    edb = inspire.EncodedDatabase(crs, db, entry_size)
    for index in (7, N + 499):
        sid, local = divmod(index, N)
        seeds, b_rows = client.query_seeded(local)
        want, want_cols = ctx.respond_nopacking(ctx.encode_shard(db, entry_size, sid), ctx.expand_rgsw(seeds, b_rows),
                                                with_columns=True)
        q = inspire.SeededClientQuery(sid, seeds, b_rows)
        full = inspire.respond_seeded(crs, edb, q)
        assert len(full.column_ciphertexts) == gamma
        assert np.array_equal(np.stack([full.ciphertext.a, full.ciphertext.b]), want)
        assert np.array_equal(np.stack([np.stack([c.a, c.b]) for c in full.column_ciphertexts]), want_cols)
        comb = inspire.respond_seeded(crs, edb, q, with_columns=False)
        assert np.array_equal(np.stack([comb.ciphertext.a, comb.ciphertext.b]), want)
    edb.close()
    crs.close()
    with pytest.raises(inspire.PirError, match="num_columns"):
        inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 3, mode="crt_fixed")
