"""The serving loop (continuous batching over several streams, mixed
databases, shards and clients): every response equals the one the same
query gets alone, and the oracle's for sampled queries; backpressure, ticket
and error behaviour."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(11, 43))


@pytest.fixture(scope="module")
def world(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(99)
    ctx = O.Ctx()
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    sizes = [2 * N + 700, N // 2, 4 * N]  # databases of different sizes
    raws = [rng.integers(0, 256, size=s * ENTRY, dtype=np.uint8) for s in sizes]
    dbs = [inspire.EncodedDatabase(crs, r, ENTRY) for r in raws]
    clients = [O.Client(ctx, seed=s, rng_seed=200 + s) for s in range(3)]
    ids, ybodies = [], []
    for c in clients:
        yb, _ = c.packing_keys(pack)
        ybodies.append(yb)
        ids.append(crs.register_client(inspire.ClientPackingKeys(y_body=yb)))
    return dict(O=O, inspire=inspire, ctx=ctx, crs=crs, pack=pack, raws=raws, dbs=dbs, sizes=sizes,
                clients=clients, ids=ids, ybodies=ybodies, rng=rng)


def make_queries(W, n):
    rng = W["rng"]
    qs = []
    for _ in range(n):
        d = int(rng.integers(0, len(W["dbs"])))
        idx = int(rng.integers(0, W["sizes"][d]))
        c = int(rng.integers(0, len(W["clients"])))
        seeds, b_rows = W["clients"][c].query_seeded(idx % N)
        qs.append(dict(db=d, shard=idx // N, idx=idx, client=c, seeds=seeds, b_rows=b_rows))
    return qs


def alone(W, q):
    inspire = W["inspire"]
    return inspire.respond_seeded_batch(W["crs"], W["dbs"][q["db"]], [q["shard"]], q["seeds"][None],
                                        q["b_rows"][None], [W["ids"][q["client"]]])[0]


def test_served_equals_alone_under_concurrency(world):
    W = world
    inspire = W["inspire"]
    qs = make_queries(W, 240)
    want = [alone(W, q) for q in qs]
    srv = inspire.Server(W["crs"], max_batch=32, max_inflight=3, capacity=96)
    tickets = [None] * len(qs)
    errors = []

    def submitter(part):
        rng = np.random.default_rng(part)
        order = list(range(part, len(qs), 3))
        k = 0
        while k < len(order):
            burst = order[k:k + int(rng.integers(1, 24))]
            # one call per database (a submit names one database)
            by_db = {}
            for i in burst:
                by_db.setdefault(qs[i]["db"], []).append(i)
            for d, idxs in by_db.items():
                pos = 0
                while pos < len(idxs):
                    sub = idxs[pos:]
                    t, rc = srv.submit(W["dbs"][d], [qs[i]["shard"] for i in sub],
                                       np.stack([qs[i]["seeds"] for i in sub]),
                                       np.stack([qs[i]["b_rows"] for i in sub]),
                                       [W["ids"][qs[i]["client"]] for i in sub])
                    for j, tk in enumerate(t):
                        tickets[sub[j]] = int(tk)
                    pos += len(t)
                    if rc == inspire.pir.nat.ERR_BUSY:
                        threading.Event().wait(0.001)  # capacity reached: let the collector drain
                    elif rc != 0:
                        errors.append(rc)
                        return
            k += len(burst)

    got = [None] * len(qs)

    def collector():
        remaining = set(range(len(qs)))
        while remaining:
            for i in sorted(remaining):
                if tickets[i] is None:
                    continue
                out = np.zeros((2, 2 * N), dtype=np.uint64)
                if srv.poll(tickets[i], out, timeout_us=200) is not None:
                    got[i] = out
                    remaining.discard(i)

    threads = [threading.Thread(target=submitter, args=(p,)) for p in range(3)]
    col = threading.Thread(target=collector)
    for t in threads:
        t.start()
    col.start()
    for t in threads:
        t.join(120)
    col.join(120)
    assert not errors
    assert not col.is_alive()
    for i in range(len(qs)):
        assert np.array_equal(got[i], want[i]), f"query {i} differs from its alone response"
    st = srv.stats()
    assert st["completed"] == len(qs) and st["submitted"] == len(qs)
    assert st["batches"] >= len(qs) // 32 and st["streams"] == 3
    srv.close()


def test_served_matches_oracle_and_decrypts(world):
    W = world
    inspire, ctx = W["inspire"], W["ctx"]
    srv = inspire.Server(W["crs"], max_batch=8, max_inflight=2, capacity=16)
    for q in make_queries(W, 3):
        t, rc = srv.submit(W["dbs"][q["db"]], [q["shard"]], q["seeds"][None], q["b_rows"][None],
                           [W["ids"][q["client"]]])
        assert rc == 0 and len(t) == 1
        out = np.zeros((2, 2 * N), dtype=np.uint64)
        assert srv.poll(int(t[0]), out) is not None
        shard = ctx.encode_shard(W["raws"][q["db"]], ENTRY, q["shard"])
        want = ctx.respond_inspiring(shard, ctx.expand_rgsw(q["seeds"], q["b_rows"]), W_SEED,
                                     mode=W["O"].MODE_CRT_FIXED, pack=W["pack"], y_body=W["ybodies"][q["client"]])
        assert np.array_equal(out, want)
        entry = W["clients"][q["client"]].extract_inspiring(out, ENTRY)
        assert np.array_equal(entry, W["raws"][q["db"]][q["idx"] * ENTRY:(q["idx"] + 1) * ENTRY])
    srv.close()


def test_serving_errors_and_tickets(world):
    W = world
    inspire = W["inspire"]
    srv = inspire.Server(W["crs"], max_batch=4, max_inflight=1, capacity=4)
    q = make_queries(W, 1)[0]
    seeds = np.stack([q["seeds"]] * 2)
    brows = np.stack([q["b_rows"]] * 2)
    db = W["dbs"][0]
    # the first query is accepted, the second names a missing shard
    t, rc = srv.submit(db, [0, 9], seeds, brows, [W["ids"][0]] * 2)
    assert len(t) == 1 and rc == inspire.pir.nat.ERR_SHARD_NOT_FOUND
    with pytest.raises(inspire.PirError, match="Shard 9 not found"):
        srv.submit(db, [9], seeds[:1], brows[:1], [W["ids"][0]])
    with pytest.raises(inspire.PirError, match="keys missing"):
        srv.submit(db, [0], seeds[:1], brows[:1], [77])
    assert srv.poll(int(t[0])) is not None
    with pytest.raises(inspire.PirError, match="ticket"):
        srv.poll(int(t[0]))  # consumed
    # capacity: 4 accepted, the fifth is refused with BUSY until polled
    five = np.stack([q["seeds"]] * 5), np.stack([q["b_rows"]] * 5)
    t, rc = srv.submit(db, [0] * 5, five[0], five[1], [W["ids"][1]] * 5)
    assert len(t) == 4 and rc == inspire.pir.nat.ERR_BUSY
    outs = []
    for tk in t:
        o = np.zeros((2, 2 * N), dtype=np.uint64)
        assert srv.poll(int(tk), o) is not None
        outs.append(o)
    assert all(np.array_equal(outs[0], o) for o in outs)
    assert srv.stats()["pending"] == 0
    srv.close()


def test_device_budget_limits_streams(world):
    W = world
    inspire = W["inspire"]
    # in-flight device memory per batch: one 152-byte descriptor per query
    # (96 bytes of seeds inline; the rows and responses stay in pinned host
    # memory)
    one_batch = 8 * 152
    srv = inspire.Server(W["crs"], max_batch=8, max_inflight=4, capacity=32, device_budget=2 * one_batch + 10)
    assert srv.stats()["streams"] == 2
    srv.close()
    with pytest.raises(inspire.PirError, match="below one batch"):
        inspire.Server(W["crs"], max_batch=8, max_inflight=4, capacity=32, device_budget=one_batch - 1)


def test_borrowed_rows_mixed_databases_one_call(world):
    """One submit naming three databases, rows read in place from pinned
    memory (no host copy): each response equals the query's alone response."""
    W = world
    inspire = W["inspire"]
    qs = make_queries(W, 40)
    want = [alone(W, q) for q in qs]
    sb = inspire.PinnedBuffer((len(qs), 6, 32), np.uint8)
    bb = inspire.PinnedBuffer((len(qs), 6, 2 * N), np.uint64)
    for i, q in enumerate(qs):
        sb.array[i], bb.array[i] = q["seeds"], q["b_rows"]
    srv = inspire.Server(W["crs"], max_batch=16, max_inflight=2, capacity=64)
    t, rc = srv.submit([W["dbs"][q["db"]] for q in qs], [q["shard"] for q in qs], sb.array, bb.array,
                       [W["ids"][q["client"]] for q in qs], borrow=True)
    assert rc == 0 and len(t) == len(qs)
    out = np.zeros((len(qs), 2, 2 * N), dtype=np.uint64)
    done = srv.poll_batch(t, out)
    assert len(done) == len(qs)
    for i in range(len(qs)):
        assert np.array_equal(out[i], want[i])
    # borrowing pageable memory is refused
    with pytest.raises(inspire.PirError, match="page-locked"):
        srv.submit(W["dbs"][0], [0], np.zeros((1, 6, 32), np.uint8), np.zeros((1, 6, 2 * N), np.uint64),
                   [W["ids"][0]], borrow=True)
    srv.close()
    sb.close()
    bb.close()


@pytest.mark.parametrize("kernel", ["pair", "single"])
def test_stage_wait_running_out(world, kernel):
    """The serving variant's bounded wait for a query's rows (copied from
    pinned host memory into shared memory) made to run out at once
    (stage_wait_iters = 0): every query of the batch fails with a device
    status after the kernel has drained its copies, the context stays
    usable, and the next batches are answered correctly.  Both Respond
    kernels: the two-CTA cluster kernel (batches up to the pair threshold;
    the two CTAs agree on the outcome before either returns) and the
    one-CTA kernel."""
    W = world
    inspire = W["inspire"]
    qs = make_queries(W, 12)
    want = [alone(W, q) for q in qs]
    old_threshold = W["crs"].pair_threshold
    W["crs"].pair_threshold = 64 if kernel == "pair" else 0
    try:
        _stage_wait_running_out(W, inspire, qs, want)
    finally:
        W["crs"].pair_threshold = old_threshold


def _stage_wait_running_out(W, inspire, qs, want):

    def serve(srv, qs):
        tickets, rc = srv.submit([W["dbs"][q["db"]] for q in qs], [q["shard"] for q in qs],
                                 np.stack([q["seeds"] for q in qs]), np.stack([q["b_rows"] for q in qs]),
                                 [W["ids"][q["client"]] for q in qs])
        assert rc == 0 and len(tickets) == len(qs)
        return tickets

    srv = inspire.Server(W["crs"], max_batch=8, max_inflight=2, capacity=32, stage_wait_iters=0)
    tickets = serve(srv, qs)
    out = np.zeros((2, 2 * N), np.uint64)
    for t in tickets:
        with pytest.raises(inspire.PirError, match="did not reach the GPU"):
            srv.poll(int(t), out)
    st = srv.stats()
    assert st["completed"] == len(qs) and st["pending"] == 0
    srv.close()
    # the same context, a server with the default bound: correct answers
    srv = inspire.Server(W["crs"], max_batch=8, max_inflight=2, capacity=32)
    for _ in range(2):
        tickets = serve(srv, qs)
        got = np.zeros((len(qs), 2, 2 * N), np.uint64)
        srv.poll_batch(tickets, got)
        for k in range(len(qs)):
            assert np.array_equal(got[k], want[k]), k
    srv.close()


def test_admission_by_device_memory(oracle_mod):
    """A context with a device budget: a database, client keys and a serving
    loop are admitted while they fit and refused with ERR_OUT_OF_MEMORY
    (before anything is allocated) when they do not; freeing returns the
    bytes; a budget below what is in use is refused; the HTTP backend evicts
    idle cached clients to make room."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire
    from inspire import _native as nat
    from inspire.http_server import GpuBackend

    O = oracle_mod
    ctx = O.Ctx()
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    base, budget = crs.device_memory()
    assert base > 0 and budget == 0
    db = np.random.default_rng(8).integers(0, 256, size=2 * N * ENTRY, dtype=np.uint8)  # 2 shards
    key_bytes = 3 * 2 * N * 4  # one client's body table
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    used0, _ = crs.device_memory()
    assert used0 >= base + 2 * (16 * N * 2 + 2 * 3 * 16 * N * 4)  # raw columns + contracted form
    # room for the key upload buffer, the client table and three clients' keys
    crs.set_device_budget(used0 + 3 * 2 * N * 8 + 256 * 8 + 3 * key_bytes + 1024)
    with pytest.raises(inspire.PirError, match="does not fit the device budget") as ei:
        inspire.EncodedDatabase(crs, db, ENTRY)
    assert ei.value.status == nat.ERR_OUT_OF_MEMORY
    assert crs.device_memory()[0] == used0  # nothing of the refused database stays reserved
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    clients = [O.Client(ctx, seed=50 + s, rng_seed=500 + s) for s in range(8)]
    ybs = [c.packing_keys(pack)[0] for c in clients]
    ids = []
    with pytest.raises(inspire.PirError) as ei:
        for yb in ybs:
            ids.append(crs.register_client(inspire.ClientPackingKeys(y_body=yb)))
    assert ei.value.status == nat.ERR_OUT_OF_MEMORY and len(ids) == 3
    used, budget = crs.device_memory()
    assert used <= budget
    with pytest.raises(inspire.PirError, match="below"):
        crs.set_device_budget(used - 1)
    # freeing returns the bytes: another client fits again
    crs.release_client(ids.pop())
    ids.append(crs.register_client(inspire.ClientPackingKeys(y_body=ybs[3])))
    # a serving loop needs slot buffers: refused while the budget is full
    with pytest.raises(inspire.PirError) as ei:
        inspire.Server(crs, max_batch=1024, max_inflight=64, capacity=4096)
    assert ei.value.status == nat.ERR_OUT_OF_MEMORY
    # the admitted clients answer correctly (without a budget: the call's
    # staging buffers need room too)
    crs.set_device_budget(0)
    seeds, b_rows = clients[3].query_seeded(77)
    out = inspire.respond_seeded_batch(crs, edb, [1], seeds[None], b_rows[None], [ids[-1]])
    assert np.array_equal(clients[3].extract_inspiring(out[0], ENTRY), db[(N + 77) * ENTRY:(N + 78) * ENTRY])
    for i in ids:
        crs.release_client(i)
    # the HTTP backend's client cache makes room by evicting idle clients
    crs.set_device_budget(0)
    backend = GpuBackend(crs, edb, max_batch=8, max_inflight=1, capacity=16)
    used, _ = crs.device_memory()
    crs.set_device_budget(used + 2 * key_bytes + 4096)
    for k, c in enumerate(clients[:6]):
        yb = ybs[k]
        s, b = c.query_seeded(k)
        got = backend.respond_seeded_inspiring(inspire.SeededClientQuery(
            0, s, b, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=yb)))
        assert np.array_equal(c.extract_inspiring(got, ENTRY), db[k * ENTRY:(k + 1) * ENTRY])
    assert len(backend._keys) <= 2
    backend.close()
    edb.close()
    crs.close()


def test_native_open_loop_driver(world):
    """Server.drive (inspire_server_drive): queries submitted at their
    arrival times by the library's own threads, through backpressure (more
    queries than slots); every query is submitted no earlier than its arrival
    and completes after it, and the kept responses equal the queries'
    responses alone."""
    W = world
    inspire = W["inspire"]
    from inspire.pir import now_ns

    qs = make_queries(W, 8)
    want = [alone(W, q) for q in qs]
    pool_seeds = np.ascontiguousarray(np.stack([q["seeds"] for q in qs]))
    pool_rows = np.ascontiguousarray(np.stack([q["b_rows"] for q in qs]))
    n = 3000
    srv = inspire.Server(W["crs"], max_batch=64, max_inflight=4, capacity=256)
    try:
        handles = np.array([srv.handle_of(W["dbs"][qs[k % 8]["db"]]) for k in range(n)], dtype=np.uint64)
        shards = np.array([qs[k % 8]["shard"] for k in range(n)], dtype=np.uint32)
        cids = np.array([W["ids"][qs[k % 8]["client"]] for k in range(n)], dtype=np.int32)
        gaps = np.random.default_rng(5).exponential(1e9 / 200_000, size=n).astype(np.int64)  # ~200 K q/s
        arrivals = now_ns() + 5_000_000 + np.cumsum(gaps)
        sub, done, kept = srv.drive(handles, shards, cids, pool_seeds, pool_rows, arrivals, n_keep=16)
        assert (sub >= arrivals).all() and (done >= arrivals).all()
        for k in range(16):
            assert np.array_equal(kept[k], want[k % 8]), k
        st = srv.stats()
        assert st["completed"] == n and st["pending"] == 0
        # borrowed rows from page-locked memory
        ps = inspire.PinnedBuffer(pool_seeds.shape, np.uint8)
        pr = inspire.PinnedBuffer(pool_rows.shape, np.uint64)
        ps.array[:] = pool_seeds
        pr.array[:] = pool_rows
        arrivals = now_ns() + 2_000_000 + np.cumsum(gaps[:500])
        _, done, kept = srv.drive(handles[:500], shards[:500], cids[:500], ps.array, pr.array, arrivals, borrow=True,
                                  n_keep=8)
        assert (done >= arrivals).all()
        for k in range(8):
            assert np.array_equal(kept[k], want[k]), k
        ps.close()
        pr.close()
    finally:
        srv.close()


def test_native_driver_stops_on_an_invalid_query(world):
    """A query naming a missing shard in the middle of a driven stream ends
    Server.drive with the crate's error, promptly (the collector stops too),
    and the server keeps answering afterwards."""
    import time

    W = world
    inspire = W["inspire"]
    from inspire.pir import now_ns

    qs = make_queries(W, 4)
    want = alone(W, qs[0])
    pool_seeds = np.ascontiguousarray(np.stack([q["seeds"] for q in qs]))
    pool_rows = np.ascontiguousarray(np.stack([q["b_rows"] for q in qs]))
    n = 400
    srv = inspire.Server(W["crs"], max_batch=32, max_inflight=2, capacity=128)
    try:
        handles = np.array([srv.handle_of(W["dbs"][qs[k % 4]["db"]]) for k in range(n)], dtype=np.uint64)
        shards = np.array([qs[k % 4]["shard"] for k in range(n)], dtype=np.uint32)
        shards[150] = 10_000  # no such shard in any database
        cids = np.array([W["ids"][qs[k % 4]["client"]] for k in range(n)], dtype=np.int32)
        arrivals = now_ns() + 2_000_000 + np.arange(n, dtype=np.int64) * 5_000
        t0 = time.monotonic()
        with pytest.raises(inspire.PirError, match="not found"):
            srv.drive(handles, shards, cids, pool_seeds, pool_rows, arrivals)
        assert time.monotonic() - t0 < 10.0
        st = srv.stats()  # every accepted query was collected
        assert st["pending"] == 0 and st["submitted"] == st["completed"] == 150
        t, rc = srv.submit(W["dbs"][qs[0]["db"]], [qs[0]["shard"]], qs[0]["seeds"][None], qs[0]["b_rows"][None],
                           [W["ids"][qs[0]["client"]]])
        assert rc == 0
        out = np.zeros((1, 2, 2 * N), dtype=np.uint64)
        assert len(srv.poll_batch(t, out)) == 1 and np.array_equal(out[0], want)
    finally:
        srv.close()


@pytest.mark.gpu
def test_native_driver_collects_every_query_after_a_device_failure(world):
    """Every driven query fails on the device (the rows' bounded wait set to
    run out at once): Server.drive ends with the device status of the first
    failure, and every query submitted before the submitter stopped has been
    collected, so that no record is left occupied in the server."""
    W = world
    inspire = W["inspire"]
    from inspire.pir import now_ns

    qs = make_queries(W, 4)
    pool_seeds = np.ascontiguousarray(np.stack([q["seeds"] for q in qs]))
    pool_rows = np.ascontiguousarray(np.stack([q["b_rows"] for q in qs]))
    n = 300
    srv = inspire.Server(W["crs"], max_batch=16, max_inflight=2, capacity=64, stage_wait_iters=0)
    try:
        handles = np.array([srv.handle_of(W["dbs"][qs[k % 4]["db"]]) for k in range(n)], dtype=np.uint64)
        shards = np.array([qs[k % 4]["shard"] for k in range(n)], dtype=np.uint32)
        cids = np.array([W["ids"][qs[k % 4]["client"]] for k in range(n)], dtype=np.int32)
        arrivals = now_ns() + 2_000_000 + np.arange(n, dtype=np.int64) * 5_000
        with pytest.raises(inspire.PirError, match="did not reach the GPU|batch dropped"):
            srv.drive(handles, shards, cids, pool_seeds, pool_rows, arrivals)
        st = srv.stats()
        assert st["pending"] == 0 and st["inflight_batches"] == 0
        assert 0 < st["submitted"] == st["completed"] <= n
    finally:
        srv.close()
