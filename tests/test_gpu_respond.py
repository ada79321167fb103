"""GPU parity of the Respond path through the C ABI, bit-exact against the
oracle restatement of respond_seeded_inspiring / respond_inspiring
(src/pir/respond.rs:284-398), in both automorphism modes, plus the crate's
error behaviour and end-to-end extraction (tests/e2e_pir.rs:464-535)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(7, 39))


@pytest.fixture(scope="module")
def world(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(2024)
    n_entries = 2 * N + 900  # three shards, the last one partial
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    ctx = O.Ctx()
    client = O.Client(ctx, seed=0, rng_seed=17)
    w = {}
    for mode, omode in (("crt_fixed", O.MODE_CRT_FIXED), ("compat", O.MODE_COMPAT)):
        crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode=mode)
        edb = inspire.EncodedDatabase(crs, db, ENTRY)
        pack = O.Pack(ctx, 16, W_SEED, mode=omode)
        w[mode] = (crs, edb, pack, omode)
    shards = [ctx.encode_shard(db, ENTRY, s) for s in range(3)]
    return dict(O=O, inspire=inspire, ctx=ctx, client=client, db=db, w=w, shards=shards, n_entries=n_entries)


def oracle_response(W, mode, shard_id, rgsw, y_body=None, y_all=None):
    crs, edb, pack, omode = W["w"][mode]
    return W["ctx"].respond_inspiring(W["shards"][shard_id], rgsw, W_SEED, mode=omode, pack=pack,
                                      y_body=y_body, y_all=y_all)


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
@pytest.mark.parametrize("index", [0, 1, 2047, 2048, 4096 + 899])
def test_seeded_respond_bit_exact(world, mode, index):
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    crs, edb, pack, omode = W["w"][mode]
    sid, local = divmod(index, N)
    seeds, b_rows = client.query_seeded(local)
    y_body, _ = client.packing_keys(pack)
    want = oracle_response(W, mode, sid, ctx.expand_rgsw(seeds, b_rows), y_body=y_body)
    q = inspire.SeededClientQuery(sid, seeds, b_rows, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=y_body))
    resp = inspire.respond_seeded_inspiring(crs, edb, q)
    assert resp.column_ciphertexts == []
    assert np.array_equal(resp.ciphertext.a, want[0])
    assert np.array_equal(resp.ciphertext.b, want[1])
    got_entry = client.extract_inspiring(want, ENTRY)
    expect = W["db"][index * ENTRY:(index + 1) * ENTRY]
    if mode == "crt_fixed":
        assert np.array_equal(got_entry, expect)


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_in_process_y_all_keys(world, mode):
    """Queries built in-process carry y_all (inspiring2.rs:670-695); respond
    uses it instead of rotating y_body (respond.rs:365-377)."""
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    crs, edb, pack, omode = W["w"][mode]
    seeds, b_rows = client.query_seeded(321)
    y_body, y_all = client.packing_keys(pack)
    want = oracle_response(W, mode, 1, ctx.expand_rgsw(seeds, b_rows), y_all=y_all)
    q = inspire.SeededClientQuery(1, seeds, b_rows,
                                  inspiring_packing_keys=inspire.ClientPackingKeys(y_body=y_body, y_all=y_all))
    resp = inspire.respond_seeded_inspiring(crs, edb, q)
    assert np.array_equal(np.stack([resp.ciphertext.a, resp.ciphertext.b]), want)


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_unseeded_respond_inspiring(world, mode):
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    crs, edb, pack, omode = W["w"][mode]
    seeds, b_rows = client.query_seeded(1000)
    rgsw = ctx.expand_rgsw(seeds, b_rows)
    y_body, _ = client.packing_keys(pack)
    want = oracle_response(W, mode, 2, rgsw, y_body=y_body)
    q = inspire.ClientQuery(2, rgsw, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=y_body))
    resp = inspire.respond_inspiring(crs, edb, q)
    assert np.array_equal(np.stack([resp.ciphertext.a, resp.ciphertext.b]), want)


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_batch_equals_single(world, mode):
    """A batch mixing shards and clients returns, per query, the single-query
    response."""
    W = world
    inspire, ctx, O = W["inspire"], W["ctx"], W["O"]
    crs, edb, pack, omode = W["w"][mode]
    clients = [O.Client(ctx, seed=s, rng_seed=100 + s) for s in range(3)]
    ids, keys = [], []
    for c in clients:
        yb, _ = c.packing_keys(pack)
        keys.append(yb)
        ids.append(crs.register_client(inspire.ClientPackingKeys(y_body=yb)))
    idxs = [5, 2050, 4100, 77, 4995, 2047]
    seeds = np.zeros((len(idxs), 6, 32), dtype=np.uint8)
    brows = np.zeros((len(idxs), 6, 2 * N), dtype=np.uint64)
    sids, cids = [], []
    for k, ix in enumerate(idxs):
        c = k % 3
        s, b = clients[c].query_seeded(ix % N)
        seeds[k], brows[k] = s, b
        sids.append(ix // N)
        cids.append(ids[c])
    out = inspire.respond_seeded_batch(crs, edb, sids, seeds, brows, cids)
    for k in range(len(idxs)):
        q = inspire.SeededClientQuery(sids[k], seeds[k], brows[k],
                                      inspiring_packing_keys=inspire.ClientPackingKeys(y_body=keys[k % 3]))
        r = inspire.respond_seeded_inspiring(crs, edb, q)
        assert np.array_equal(out[k], np.stack([r.ciphertext.a, r.ciphertext.b]))
    want0 = oracle_response(W, mode, sids[0], ctx.expand_rgsw(seeds[0], brows[0]), y_body=keys[0])
    assert np.array_equal(out[0], want0)
    for i in ids:
        crs.release_client(i)


def test_errors_follow_reference(world):
    W = world
    inspire, client = W["inspire"], W["client"]
    crs, edb, pack, _ = W["w"]["crt_fixed"]
    seeds, b_rows = client.query_seeded(3)
    y_body, _ = client.packing_keys(pack)
    keys = inspire.ClientPackingKeys(y_body=y_body)
    with pytest.raises(inspire.PirError, match="Shard 3 not found"):
        inspire.respond_seeded_inspiring(crs, edb, inspire.SeededClientQuery(3, seeds, b_rows, inspiring_packing_keys=keys))
    with pytest.raises(inspire.PirError, match="InspiRING client packing keys missing from query"):
        inspire.respond_seeded_inspiring(crs, edb, inspire.SeededClientQuery(0, seeds, b_rows))
    with pytest.raises(inspire.PirError, match="y_all and y_body are both empty"):
        inspire.respond_seeded_inspiring(crs, edb, inspire.SeededClientQuery(
            0, seeds, b_rows, inspiring_packing_keys=inspire.ClientPackingKeys()))
    # keys-missing is checked before the shard lookup (respond.rs:296-305)
    with pytest.raises(inspire.PirError, match="keys missing"):
        inspire.respond_seeded_inspiring(crs, edb, inspire.SeededClientQuery(99, seeds, b_rows))


@pytest.mark.parametrize("entry_size,gamma", [(2, 1), (8, 4), (16, 8)])
def test_other_column_counts(oracle_mod, entry_size, gamma):
    torch = pytest.importorskip("torch")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(entry_size)
    n_entries = 1500
    db = rng.integers(0, 256, size=n_entries * entry_size, dtype=np.uint8)
    ctx = O.Ctx()
    client = O.Client(ctx, seed=1, rng_seed=entry_size)
    for mode, omode in (("crt_fixed", O.MODE_CRT_FIXED), ("compat", O.MODE_COMPAT)):
        crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, gamma, mode=mode)
        edb = inspire.EncodedDatabase(crs, db, entry_size)
        pack = O.Pack(ctx, gamma, W_SEED, mode=omode)
        seeds, b_rows = client.query_seeded(1234)
        y_body, _ = client.packing_keys(pack)
        want = ctx.respond_inspiring(ctx.encode_shard(db, entry_size, 0), ctx.expand_rgsw(seeds, b_rows), W_SEED,
                                     mode=omode, pack=pack, y_body=y_body)
        q = inspire.SeededClientQuery(0, seeds, b_rows, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=y_body))
        default = crs.pair_threshold
        for thr in (default, 0):  # the two-CTA cluster kernel, then one CTA per query
            crs.pair_threshold = thr
            r = inspire.respond_seeded_inspiring(crs, edb, q)
            assert np.array_equal(np.stack([r.ciphertext.a, r.ciphertext.b]), want), (mode, thr)
        # the serving loop's variant of the one-CTA kernel (rows read from
        # page-locked host memory)
        cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
        srv = inspire.Server(crs, max_batch=8, max_inflight=1, capacity=8)
        try:
            t, rc = srv.submit(edb, [0, 0], np.stack([seeds, seeds]), np.stack([b_rows, b_rows]), [cid, cid])
            assert rc == 0 and len(t) == 2
            out = np.zeros((2, 2, 2 * N), dtype=np.uint64)
            assert len(srv.poll_batch(t, out)) == 2
            assert np.array_equal(out[0], want) and np.array_equal(out[1], want), mode
        finally:
            srv.close()
            crs.pair_threshold = default
        if mode == "crt_fixed":
            assert np.array_equal(client.extract_inspiring(want, entry_size),
                                  db[1234 * entry_size:1235 * entry_size])


def test_full_size_database_extracts(oracle_mod):
    """2^20 entries x 32 B resident (512 shards): sampled queries decrypt to
    their entries (crt_fixed) and the first matches the oracle bit for bit."""
    torch = pytest.importorskip("torch")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(20)
    n_entries = 1 << 20
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    ctx = O.Ctx()
    client = O.Client(ctx, seed=2, rng_seed=21)
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    assert edb.num_shards == 512
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    y_body, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
    idxs = rng.integers(0, n_entries, size=24)
    seeds = np.zeros((len(idxs), 6, 32), dtype=np.uint8)
    brows = np.zeros((len(idxs), 6, 2 * N), dtype=np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = client.query_seeded(int(ix) % N)
    out = inspire.respond_seeded_batch(crs, edb, [int(i) // N for i in idxs], seeds, brows, [cid] * len(idxs))
    for k, ix in enumerate(idxs):
        ix = int(ix)
        assert np.array_equal(client.extract_inspiring(out[k], ENTRY), db[ix * ENTRY:(ix + 1) * ENTRY])
    ix = int(idxs[0])
    want = ctx.respond_inspiring(ctx.encode_shard(db, ENTRY, ix // N), ctx.expand_rgsw(seeds[0], brows[0]), W_SEED,
                                 mode=O.MODE_CRT_FIXED, pack=pack, y_body=y_body)
    assert np.array_equal(out[0], want)


def test_extract_inspiring_device(world):
    """decrypt + extract_inspiring on the device (extract.rs:155-182) equals
    the oracle's extraction and recovers the queried entries."""
    W = world
    torch = pytest.importorskip("torch")
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    crs, edb, pack, omode = W["w"]["crt_fixed"]
    y_body, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
    idxs = [0, 5, 2047, 2048, 4096 + 899, 3000]
    seeds = np.zeros((len(idxs), 6, 32), np.uint8)
    brows = np.zeros((len(idxs), 6, 2 * N), np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = client.query_seeded(ix % N)
    out = inspire.respond_seeded_batch(crs, edb, [ix // N for ix in idxs], seeds, brows, [cid] * len(idxs))
    dev = torch.device("cuda", 0)
    d_ct = torch.from_numpy(out.view(np.int64)).to(dev)
    d_sk = torch.from_numpy(np.ascontiguousarray(client.sk).view(np.int64)).to(dev)
    for entry in (ENTRY, 31, 7):
        d_e = torch.zeros((len(idxs), entry), dtype=torch.uint8, device=dev)
        inspire.pir.extract_inspiring_device(crs, d_sk.data_ptr(), d_ct.data_ptr(), len(idxs), entry, d_e.data_ptr(),
                                             torch.cuda.current_stream(dev).cuda_stream)
        got = d_e.cpu().numpy()
        for k, ix in enumerate(idxs):
            want = client.extract_inspiring(out[k], entry)
            assert np.array_equal(got[k], want)
            if entry == ENTRY:
                assert np.array_equal(got[k], W["db"][ix * ENTRY:(ix + 1) * ENTRY])
    crs.release_client(cid)


def test_batch_device_call_in_cuda_graph(world):
    """The device-buffer batch call makes no configuration call or copy, so
    it can be captured in a CUDA graph; replays return the same responses."""
    W = world
    torch = pytest.importorskip("torch")
    inspire, client = W["inspire"], W["client"]
    crs, edb, pack, omode = W["w"]["crt_fixed"]
    y_body, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
    idxs = [1, 2049, 4100, 77]
    n = len(idxs)
    seeds = np.zeros((n, 6, 32), np.uint8)
    brows = np.zeros((n, 6, 2 * N), np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = client.query_seeded(ix % N)
    want = inspire.respond_seeded_batch(crs, edb, [ix // N for ix in idxs], seeds, brows, [cid] * n)
    dev = torch.device("cuda", 0)
    d_sid = torch.tensor([ix // N for ix in idxs], dtype=torch.int32, device=dev)
    d_seeds = torch.from_numpy(np.ascontiguousarray(seeds[:, 3:6])).to(dev)
    d_brows = torch.from_numpy(np.ascontiguousarray(brows[:, 3:6]).view(np.int64)).to(dev)
    d_cid = torch.full((n,), cid, dtype=torch.int32, device=dev)
    d_out = torch.zeros((n, 2, 2 * N), dtype=torch.int64, device=dev)
    d_st = torch.zeros(n, dtype=torch.int32, device=dev)
    s = torch.cuda.Stream(dev)

    def call(stream):
        inspire.respond_seeded_batch_device(crs, edb, n, d_sid.data_ptr(), d_seeds.data_ptr(), d_brows.data_ptr(),
                                            d_cid.data_ptr(), d_out.data_ptr(), d_st.data_ptr(), stream.cuda_stream)

    with torch.cuda.stream(s):
        call(s)  # warm-up outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        call(s)
    d_out.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert not d_st.cpu().numpy().any()
    assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want)
    crs.release_client(cid)


def test_unseeded_batch_equals_single(world):
    """Batched full-query respond_inspiring: each result equals the
    single-query call and the oracle."""
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    crs, edb, pack, omode = W["w"]["crt_fixed"]
    y_body, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
    idxs = [3, 2050, 4101]
    rg = np.stack([ctx.expand_rgsw(*client.query_seeded(ix % N)).reshape(6, 2, 2 * N) for ix in idxs])
    out = inspire.respond_batch(crs, edb, [ix // N for ix in idxs], rg, [cid] * len(idxs))
    for k, ix in enumerate(idxs):
        want = oracle_response(W, "crt_fixed", ix // N, rg[k].reshape(12, 2 * N), y_body=y_body)
        assert np.array_equal(out[k], want)
    crs.release_client(cid)


def test_batch_device_capped_grid(world):
    """inspire_respond_seeded_batch_device_grid: with the grid capped below
    the batch each CTA answers several queries in turn; the responses equal
    the one-CTA-per-query call's."""
    W = world
    torch = pytest.importorskip("torch")
    inspire, client = W["inspire"], W["client"]
    crs, edb, pack, omode = W["w"]["crt_fixed"]
    y_body, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
    idxs = [3, 2050, 4101, 78, 1999, 4995, 11]
    n = len(idxs)
    seeds = np.zeros((n, 6, 32), np.uint8)
    brows = np.zeros((n, 6, 2 * N), np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = client.query_seeded(ix % N)
    want = inspire.respond_seeded_batch(crs, edb, [ix // N for ix in idxs], seeds, brows, [cid] * n)
    dev = torch.device("cuda", 0)
    d_sid = torch.tensor([ix // N for ix in idxs], dtype=torch.int32, device=dev)
    d_seeds = torch.from_numpy(np.ascontiguousarray(seeds[:, 3:6])).to(dev)
    d_brows = torch.from_numpy(np.ascontiguousarray(brows[:, 3:6]).view(np.int64)).to(dev)
    d_cid = torch.full((n,), cid, dtype=torch.int32, device=dev)
    for ctas in (1, 3, 7, 100):
        d_out = torch.zeros((n, 2, 2 * N), dtype=torch.int64, device=dev)
        d_st = torch.full((n,), -1, dtype=torch.int32, device=dev)
        inspire.respond_seeded_batch_device(crs, edb, n, d_sid.data_ptr(), d_seeds.data_ptr(), d_brows.data_ptr(),
                                            d_cid.data_ptr(), d_out.data_ptr(), d_st.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream, max_ctas=ctas)
        torch.cuda.synchronize()
        assert not d_st.cpu().numpy().any(), ctas
        assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want), ctas
    crs.release_client(cid)


def test_concurrent_host_calls_on_one_context(world):
    """Several host threads calling the synchronous entry points on one
    context at once (the crate's callers hold Arc<AppState> on tokio workers):
    every result equals the one the same call returns alone."""
    import threading

    W = world
    inspire, client = W["inspire"], W["client"]
    crs, edb, pack, omode = W["w"]["crt_fixed"]
    y_body, _ = client.packing_keys(pack)
    keys = inspire.ClientPackingKeys(y_body=y_body)
    qs = []
    for k, index in enumerate((3, 2050, 4100, 777, 1999, 4096 + 898)):
        sid, local = divmod(index, N)
        seeds, b_rows = client.query_seeded(local)
        qs.append(inspire.SeededClientQuery(sid, seeds, b_rows, inspiring_packing_keys=keys))

    def call(kind, q):
        if kind == 0:
            r = inspire.respond_seeded_inspiring(crs, edb, q)
        else:
            r = inspire.respond_seeded(crs, edb, q, with_columns=(kind == 2))
        return np.concatenate([r.ciphertext.a, r.ciphertext.b])

    jobs = [(kind, k) for k in range(len(qs)) for kind in range(3)]
    alone = {j: call(j[0], qs[j[1]]) for j in jobs}
    got, errors = {}, []

    def worker(t):
        try:
            for rep in range(3):
                for j in jobs[t::4]:
                    got[(j, rep, t)] = call(j[0], qs[j[1]])
        except BaseException as e:  # reported below
            errors.append(e)

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    assert not errors, errors
    assert len(got) == 3 * len(jobs)
    for (j, rep, t), v in got.items():
        assert np.array_equal(v, alone[j]), (j, rep, t)


def test_batch_from_page_locked_buffers(world):
    """respond_seeded_batch with page-locked rows and responses: the kernel
    reads the rows in place and writes the responses straight to host memory;
    the results equal the staged call's, and both modes match the oracle."""
    W = world
    inspire, ctx, client = W["inspire"], W["ctx"], W["client"]
    idxs = [5, 2048 + 17, 4096 + 898, 1024, 3000]
    for mode in ("crt_fixed", "compat"):
        crs, edb, pack, omode = W["w"][mode]
        y_body, _ = client.packing_keys(pack)
        cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
        n = len(idxs)
        seeds = inspire.pir.PinnedBuffer((n, 6, 32), np.uint8)
        rows = inspire.pir.PinnedBuffer((n, 6, 2 * N), np.uint64)
        out = inspire.pir.PinnedBuffer((n, 2, 2 * N), np.uint64)
        sids = []
        for k, index in enumerate(idxs):
            sid, local = divmod(index, N)
            seeds.array[k], rows.array[k] = client.query_seeded(local)
            sids.append(sid)
        staged = inspire.respond_seeded_batch(crs, edb, sids, seeds.array.copy(), rows.array.copy(), [cid] * n)
        out.array[...] = 0
        got = inspire.respond_seeded_batch(crs, edb, sids, seeds.array, rows.array, [cid] * n, out=out.array)
        assert got is out.array and np.array_equal(got, staged)
        k = 2
        want = oracle_response(W, mode, sids[k], ctx.expand_rgsw(seeds.array[k], rows.array[k]), y_body=y_body)
        assert np.array_equal(got[k, 0], want[0]) and np.array_equal(got[k, 1], want[1])
        with pytest.raises(inspire.PirError, match="Shard 9 not found"):
            inspire.respond_seeded_batch(crs, edb, [0, 9, 0, 0, 0], seeds.array, rows.array, [cid] * n,
                                         out=out.array)
        for b in (seeds, rows, out):
            b.close()
        crs.release_client(cid)


def test_carried_keys_reuse_one_table(world):
    """Queries that carry their packing keys rebuild them into one table the
    context keeps: consecutive calls switching clients and between the y_body
    and y_all forms, a client registration in between and a CRS reload (which
    frees every key table) each answer as the oracle does."""
    import ctypes as C

    W = world
    inspire, ctx, O = W["inspire"], W["ctx"], W["O"]
    crs, edb, pack, omode = W["w"]["crt_fixed"]
    clients = [W["client"], O.Client(ctx, seed=5, rng_seed=9)]
    keys = [c.packing_keys(pack) for c in clients]

    def call(k, form, index):
        sid, local = divmod(index, N)
        seeds, b_rows = clients[k].query_seeded(local)
        yb, ya = keys[k]
        pk = inspire.ClientPackingKeys(y_body=yb) if form == "body" else inspire.ClientPackingKeys(y_all=ya)
        r = inspire.respond_seeded_inspiring(crs, edb, inspire.SeededClientQuery(sid, seeds, b_rows,
                                                                               inspiring_packing_keys=pk))
        want = oracle_response(W, "crt_fixed", sid, ctx.expand_rgsw(seeds, b_rows),
                               **({"y_body": yb} if form == "body" else {"y_all": ya}))
        assert np.array_equal(np.stack([r.ciphertext.a, r.ciphertext.b]), want), (k, form, index)

    call(0, "body", 5)
    call(1, "body", 2050)
    call(0, "all", 77)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=keys[1][0]))
    call(1, "all", 4100)
    call(1, "body", 9)
    seeds, b_rows = clients[1].query_seeded(9)
    got = inspire.respond_seeded_batch(crs, edb, [0], seeds[None], b_rows[None], [cid])[0]
    assert np.array_equal(got, oracle_response(W, "crt_fixed", 0, ctx.expand_rgsw(seeds, b_rows), y_body=keys[1][0]))
    # reload the same CRS: every key table (the carried keys' too) is freed
    seed = (C.c_uint8 * 32).from_buffer_copy(W_SEED)
    assert crs.L.inspire_crs_load(crs.h, C.cast(seed, C.c_void_p), 16) == 0
    call(0, "body", 1)
    call(1, "all", 2048)
