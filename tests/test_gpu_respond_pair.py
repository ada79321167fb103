"""The two-CTA cluster Respond kernel (one CTA per CRT residue, used for
launches of at most `pair_threshold` queries) against the one-CTA kernel and
the oracle: every call path (single query, host batch, page-locked batch,
device batch, serving loop), both automorphism modes, seeded and full
queries, body and full client key tables, and the seeded expansion's
hand-off of residue 1's stream position when residue 0 rejected draws."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(3, 35))
Q = (268369921, 249561089)


@pytest.fixture(scope="module")
def world(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(4242)
    n_entries = 3 * N + 500
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    ctx = O.Ctx()
    clients = [O.Client(ctx, seed=s, rng_seed=300 + s) for s in range(2)]
    w = {}
    for mode, omode in (("crt_fixed", O.MODE_CRT_FIXED), ("compat", O.MODE_COMPAT)):
        crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode=mode)
        edb = inspire.EncodedDatabase(crs, db, ENTRY)
        pack = O.Pack(ctx, 16, W_SEED, mode=omode)
        keys = [c.packing_keys(pack) for c in clients]
        ids = [crs.register_client(inspire.ClientPackingKeys(y_body=yb)) for yb, _ in keys]
        w[mode] = dict(crs=crs, edb=edb, pack=pack, omode=omode, keys=keys, ids=ids)
    shards = [ctx.encode_shard(db, ENTRY, s) for s in range(4)]
    return dict(O=O, inspire=inspire, ctx=ctx, clients=clients, db=db, w=w, shards=shards, rng=rng,
                default_threshold=w["crt_fixed"]["crs"].pair_threshold)


def queries(W, n, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        idx = int(rng.integers(0, W["db"].size // ENTRY))
        c = int(rng.integers(0, len(W["clients"])))
        seeds, b_rows = W["clients"][c].query_seeded(idx % N)
        out.append(dict(idx=idx, shard=idx // N, client=c, seeds=seeds, b_rows=b_rows))
    return out


def stack(qs):
    return (np.array([q["shard"] for q in qs]), np.stack([q["seeds"] for q in qs]),
            np.stack([q["b_rows"] for q in qs]))


def oracle(W, mode, q):
    M = W["w"][mode]
    rgsw = W["ctx"].expand_rgsw(q["seeds"], q["b_rows"])
    return W["ctx"].respond_inspiring(W["shards"][q["shard"]], rgsw, W_SEED, mode=M["omode"], pack=M["pack"],
                                      y_body=M["keys"][q["client"]][0])


def with_threshold(crs, t, fn):
    old = crs.pair_threshold
    crs.pair_threshold = t
    try:
        return fn()
    finally:
        crs.pair_threshold = old


def residue0_end(O, seed):
    """Index after residue 0's last accepted draw in a row's seeded stream
    (Poly::from_seed_moduli, poly.rs:251-281): residue 1 starts there."""
    rng = O.Rng(seed=bytes(seed))
    q = Q[0]
    zone = ((q << (64 - q.bit_length())) - 1) & ((1 << 64) - 1)
    got = k = 0
    while got < N:
        v = rng.next_u64()
        k += 1
        if (v * q) & ((1 << 64) - 1) <= zone:
            got += 1
    return k


def test_default_threshold_is_half_the_sms(world):
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert world["default_threshold"] == sms // 2


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_batch_both_kernels_equal_oracle(world, mode):
    W = world
    inspire = W["inspire"]
    M = W["w"][mode]
    qs = queries(W, 6, seed=1)
    sid, seeds, brows = stack(qs)
    cids = [M["ids"][q["client"]] for q in qs]
    run = lambda: inspire.respond_seeded_batch(M["crs"], M["edb"], sid, seeds, brows, cids)
    pair = with_threshold(M["crs"], 64, run)
    single = with_threshold(M["crs"], 0, run)
    assert np.array_equal(pair, single)
    for k in (0, 3, 5):
        assert np.array_equal(pair[k], oracle(W, mode, qs[k])), k


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
@pytest.mark.parametrize("threshold", [64, 0], ids=["pair", "single"])
def test_single_query_paths(world, mode, threshold):
    """respond_seeded_inspiring (keys in the query) and respond_inspiring
    (full RGSW rows), y_body and y_all key forms."""
    W = world
    inspire, ctx = W["inspire"], W["ctx"]
    M = W["w"][mode]
    q = queries(W, 1, seed=7 + threshold)[0]
    yb, ya = M["keys"][q["client"]]
    want = oracle(W, mode, q)

    def run():
        r1 = inspire.respond_seeded_inspiring(M["crs"], M["edb"], inspire.SeededClientQuery(
            q["shard"], q["seeds"], q["b_rows"], inspiring_packing_keys=inspire.ClientPackingKeys(y_body=yb)))
        rgsw = ctx.expand_rgsw(q["seeds"], q["b_rows"])
        r2 = inspire.respond_inspiring(M["crs"], M["edb"], inspire.ClientQuery(
            q["shard"], rgsw, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=yb)))
        r3 = inspire.respond_seeded_inspiring(M["crs"], M["edb"], inspire.SeededClientQuery(
            q["shard"], q["seeds"], q["b_rows"],
            inspiring_packing_keys=inspire.ClientPackingKeys(y_body=yb, y_all=ya)))
        return [np.stack([r.ciphertext.a, r.ciphertext.b]) for r in (r1, r2, r3)]

    got = with_threshold(M["crs"], threshold, run)
    assert np.array_equal(got[0], want)
    assert np.array_equal(got[1], want)
    want_all = W["ctx"].respond_inspiring(W["shards"][q["shard"]], ctx.expand_rgsw(q["seeds"], q["b_rows"]),
                                          W_SEED, mode=M["omode"], pack=M["pack"], y_all=ya)
    assert np.array_equal(got[2], want_all)


def test_residue1_stream_handoff(world):
    """Rows whose residue 0 rejected draws (so residue 1 starts past index
    2048, found by the other CTA) and rows where it did not: crt_fixed
    responses equal the oracle's and decrypt."""
    W = world
    O, inspire = W["O"], W["inspire"]
    M = W["w"]["crt_fixed"]
    qs = queries(W, 24, seed=11)
    ends = [[residue0_end(O, q["seeds"][3 + t]) for t in range(3)] for q in qs]
    shifted = [k for k, e in enumerate(ends) if max(e) > N]
    plain = [k for k, e in enumerate(ends) if max(e) == N]
    assert shifted and plain, ends
    pick = shifted[:3] + plain[:1]
    sub = [qs[k] for k in pick]
    sid, seeds, brows = stack(sub)
    got = with_threshold(M["crs"], 64, lambda: inspire.respond_seeded_batch(
        M["crs"], M["edb"], sid, seeds, brows, [M["ids"][q["client"]] for q in sub]))
    for k, q in enumerate(sub):
        want = oracle(W, "crt_fixed", q)
        assert np.array_equal(got[k], want), (pick[k], ends[pick[k]])
        ent = W["clients"][q["client"]].extract_inspiring(got[k], ENTRY)
        assert np.array_equal(ent, W["db"][q["idx"] * ENTRY:(q["idx"] + 1) * ENTRY])


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_page_locked_and_device_batches(world, mode):
    """Page-locked rows (the kernel reads them in place, serving variant) and
    device-resident rows, at the threshold and one past it."""
    import torch

    W = world
    inspire = W["inspire"]
    M = W["w"][mode]
    crs = M["crs"]
    qs = queries(W, 5, seed=23)
    sid, seeds, brows = stack(qs)
    cids = np.array([M["ids"][q["client"]] for q in qs], dtype=np.int32)
    want = with_threshold(crs, 0, lambda: inspire.respond_seeded_batch(crs, M["edb"], sid, seeds, brows, cids))
    pin_rows = inspire.pir.PinnedBuffer(brows.shape, np.uint64)
    pin_out = inspire.pir.PinnedBuffer(want.shape, np.uint64)
    pin_rows.array[:] = brows
    got = with_threshold(crs, 64, lambda: inspire.respond_seeded_batch(crs, M["edb"], sid, seeds, pin_rows.array,
                                                                        cids, out=pin_out.array))
    assert np.array_equal(got, want)
    pin_rows.close()
    pin_out.close()
    assert np.array_equal(want[0], oracle(W, mode, qs[0]))

    dev = torch.device("cuda", 0)
    for n, thr in ((4, 4), (5, 4)):  # pair at the threshold, one-CTA one past it
        d_sid = torch.tensor(sid[:n].astype(np.int64), dtype=torch.int32, device=dev)
        # the device call takes rows ELL..2ELL-1 only
        d_seeds = torch.tensor(np.ascontiguousarray(seeds[:n, 3:6]), device=dev)
        d_brows = torch.tensor(np.ascontiguousarray(brows[:n, 3:6]).view(np.int64), device=dev)
        d_cid = torch.tensor(cids[:n], device=dev)
        d_out = torch.zeros((n, 2, 2 * N), dtype=torch.int64, device=dev)
        d_status = torch.full((n,), -1, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev)

        def run():
            inspire.respond_seeded_batch_device(crs, M["edb"], n, d_sid.data_ptr(), d_seeds.data_ptr(),
                                                d_brows.data_ptr(), d_cid.data_ptr(), d_out.data_ptr(),
                                                d_status.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()

        with_threshold(crs, thr, run)
        assert (d_status.cpu().numpy() == 0).all()
        assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want[:n]), (n, thr)


def test_serving_loop_small_batches(world):
    """The serving loop's small batches run on the cluster kernel: responses
    equal the one-CTA kernel's."""
    W = world
    inspire = W["inspire"]
    M = W["w"]["crt_fixed"]
    crs = M["crs"]
    qs = queries(W, 9, seed=31)
    sid, seeds, brows = stack(qs)
    cids = [M["ids"][q["client"]] for q in qs]
    want = with_threshold(crs, 0, lambda: inspire.respond_seeded_batch(crs, M["edb"], sid, seeds, brows, cids))
    srv = inspire.Server(crs, max_batch=2, max_inflight=2, capacity=16)
    try:
        tickets, rc = srv.submit([M["edb"]] * len(qs), sid, seeds, brows, cids)
        assert rc == 0 and len(tickets) == len(qs)
        got = np.zeros((len(qs), 2, 2 * N), np.uint64)
        srv.poll_batch(tickets, got)
    finally:
        srv.close()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("gamma", [1, 4, 8])
def test_other_column_counts(oracle_mod, gamma):
    """gamma < 16 (full client key tables; gamma = 1 runs no recursion step):
    both kernels equal the oracle."""
    torch = pytest.importorskip("torch")
    import inspire

    O = oracle_mod
    entry = 2 * gamma
    rng = np.random.default_rng(gamma)
    n_entries = N + 300
    db = rng.integers(0, 256, size=n_entries * entry, dtype=np.uint8)
    ctx = O.Ctx()
    client = O.Client(ctx, seed=5, rng_seed=55)
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, gamma, mode="crt_fixed")
    edb = inspire.EncodedDatabase(crs, db, entry)
    pack = O.Pack(ctx, gamma, W_SEED, mode=O.MODE_CRT_FIXED)
    yb, ya = client.packing_keys(pack)
    seeds, b_rows = client.query_seeded(17)
    shard = ctx.encode_shard(db, entry, 0)
    want = ctx.respond_inspiring(shard, ctx.expand_rgsw(seeds, b_rows), W_SEED, mode=O.MODE_CRT_FIXED, pack=pack,
                                 y_body=yb)
    q = inspire.SeededClientQuery(0, seeds, b_rows, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=yb))
    for thr in (64, 0):
        crs.pair_threshold = thr
        r = inspire.respond_seeded_inspiring(crs, edb, q)
        assert np.array_equal(np.stack([r.ciphertext.a, r.ciphertext.b]), want), thr
