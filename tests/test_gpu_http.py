"""The HTTP front end on the GPU (src/bin/server.rs:120-236, 242-337), tested
as tests/http_inspiring.rs:80-168 does: an in-process server on 127.0.0.1:0
and real requests.  Every reply equals, byte for byte, the server JSON of
the response the C-ABI call returns for that query alone (seeded queries go
through the serving loop, several connections at once); tree packing in
compat mode (b of dimension 2 ring_dim); the crate's error replies; start-up
from a data directory (crs.json, binary shards, metadata.json)."""
import json
import threading

import numpy as np
import pytest

from http_helpers import N, ciphertext_of, full_query_body, request, seeded_query_body

pytestmark = pytest.mark.gpu

ENTRY = 32
W_SEED = bytes(range(77, 109))


@pytest.fixture(scope="module")
def world(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    ctx = O.Ctx()
    rng = np.random.default_rng(71)
    db = rng.integers(0, 256, size=(3 * N + 100) * ENTRY, dtype=np.uint8)
    clients = [O.Client(ctx, seed=s, rng_seed=700 + s) for s in range(3)]
    return dict(O=O, inspire=inspire, ctx=ctx, db=db, clients=clients)


def _reply_for(inspire, params, ct, body):
    ms = json.loads(body)["processing_time_ms"]
    resp = inspire.ServerResponse(inspire.RlweCiphertext(ct[0], ct[1]), [])
    return inspire.wire.query_response_to_json(params, resp, ms)


@pytest.mark.parametrize("impl", ["native", "python"])
def test_http_inspiring_served(world, impl):
    W = world
    O, inspire, ctx = W["O"], W["inspire"], W["ctx"]
    from inspire.http_server import GpuBackend, NativeHttpServer, PirHttpServer

    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    edb = inspire.EncodedDatabase(crs, W["db"], ENTRY)
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    keys = [c.packing_keys(pack)[0] for c in W["clients"]]
    backend = None
    if impl == "python":
        backend = GpuBackend(crs, edb, max_clients=2, max_batch=8, max_inflight=2, capacity=64)
        srv = PirHttpServer(backend).start()
    else:
        srv = NativeHttpServer(crs, edb, max_clients=2, max_batch=8, max_inflight=2, capacity=64)
    url = srv.url
    rng = np.random.default_rng(5)
    jobs = []
    for k in range(18):
        c = k % 3
        idx = int(rng.integers(0, 3 * N + 100))
        seeds, b_rows = W["clients"][c].query_seeded(idx % N)
        jobs.append((c, idx, seeds, b_rows))
    results = [None] * len(jobs)

    def worker(t):
        for k in range(t, len(jobs), 6):
            c, idx, seeds, b_rows = jobs[k]
            results[k] = request(url, "POST", "/query_seeded", seeded_query_body(idx // N, seeds, b_rows, keys[c]))

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(6)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for k, (c, idx, seeds, b_rows) in enumerate(jobs):
        st, ct, body = results[k]
        assert st == 200 and ct == "application/json", body[:300]
        q = inspire.SeededClientQuery(idx // N, seeds, b_rows,
                                      inspiring_packing_keys=inspire.ClientPackingKeys(y_body=keys[c]))
        r = inspire.respond_seeded_inspiring(crs, edb, q)
        want = np.stack([r.ciphertext.a, r.ciphertext.b])
        assert body == _reply_for(inspire, crs.params, want, body), k
        got = W["clients"][c].extract_inspiring(ciphertext_of(body), ENTRY)
        assert np.array_equal(got, W["db"][idx * ENTRY:(idx + 1) * ENTRY])
    # at most max_clients keys stay resident once nothing is in flight
    if backend is not None:
        assert len(backend._keys) <= 3
    # /query (full RGSW rows) equals respond_inspiring
    seeds, b_rows = W["clients"][1].query_seeded(300)
    rgsw = ctx.expand_rgsw(seeds, b_rows)
    st, _, body = request(url, "POST", "/query", full_query_body(2, rgsw, keys[1]))
    r = inspire.respond_inspiring(crs, edb, inspire.ClientQuery(2, rgsw.reshape(6, 2, -1),
                                  inspiring_packing_keys=inspire.ClientPackingKeys(y_body=keys[1])))
    assert st == 200 and body == _reply_for(inspire, crs.params, np.stack([r.ciphertext.a, r.ciphertext.b]), body)
    # errors
    st, _, body = request(url, "POST", "/query_seeded", seeded_query_body(0, seeds, b_rows))
    assert st == 400 and b"InspiRING packing keys missing" in body
    st, _, body = request(url, "POST", "/query_seeded", seeded_query_body(4, seeds, b_rows, keys[0]))
    assert st == 400 and json.loads(body) == {"error": "Seeded query processing failed: Shard 4 not found"}
    st, _, body = request(url, "POST", "/query", full_query_body(4, rgsw, keys[0]))
    assert st == 400 and json.loads(body) == {"error": "Query processing failed: Shard 4 not found"}
    # the crate's health and params replies
    st, _, body = request(url, "GET", "/health", ctype=None)
    assert st == 200 and body == b'{"status":"ok","version":"0.1.2"}'
    st, _, body = request(url, "GET", "/params", ctype=None)
    assert st == 200 and json.loads(body)["shard_count"] == 4 and json.loads(body)["entry_count"] == 3 * N + 100
    # extractor rejections
    st, _, body = request(url, "POST", "/query_seeded", b'{"shard_id": 1,')
    assert st == 400 and body.startswith(b"Failed to parse the request body as JSON")
    st, _, body = request(url, "POST", "/query_seeded", b'{"shard_id": 1}')
    assert st == 422 and body.startswith(b"Failed to deserialize the JSON body")
    st, _, _ = request(url, "POST", "/query_seeded", seeded_query_body(0, seeds, b_rows, keys[0]), ctype="text/plain")
    assert st == 415
    srv.close()
    if backend is not None:
        backend.close()
    edb.close()
    crs.close()


@pytest.mark.parametrize("impl", ["native", "python"])
def test_http_tree_and_data_dir(world, tmp_path, impl):
    """packing_mode "tree" on both routes (respond_seeded_packed /
    respond_one_packing), compat mode, from a data directory laid out as the
    crate's setup writes it (crs.json with Galois keys, shards/, metadata.json)."""
    W = world
    O, inspire, ctx = W["O"], W["inspire"], W["ctx"]
    from inspire.http_server import PirHttpServer

    params = inspire.InspireParams(p=1 << 16)
    client = W["clients"][0]
    galois = client.galois_keys()  # (11, 6, plen) rows [a, b] per gadget row
    kg = galois[0].reshape(3, 2, -1)
    inspire.write_crs_json(str(tmp_path / "crs.json"), params, k_g=kg, k_h=kg, galois_keys=galois.reshape(11, 3, 2, -1),
                           crs_a_vectors=np.zeros((5, 2 * N), np.uint64), inspiring_w_seed=W_SEED,
                           inspiring_v_seed=bytes(32), inspiring_num_columns=16)
    crs0 = inspire.ServerCrs(params, W_SEED, 16, mode="compat")
    crs0.load_galois_keys(galois)
    edb0 = inspire.EncodedDatabase(crs0, W["db"], ENTRY)
    (tmp_path / "shards").mkdir()
    edb0.save_shards(str(tmp_path / "shards"))
    (tmp_path / "metadata.json").write_text(json.dumps({"version": "9.9.9", "ring_dim": N, "modulus": str(params.q),
                                                        "plaintext_modulus": 65536, "entry_count": 3 * N + 100,
                                                        "shard_count": 4}))
    from inspire.http_server import NativeHttpServer

    srv = PirHttpServer.from_data_dir(str(tmp_path), params, mode="compat", mmap=True, host="127.0.0.1",
                                      port=0).start()
    py_srv = srv
    if impl == "native":
        b = srv.backend
        srv = NativeHttpServer(b.crs, b.edb, server=b.server, crs_json=b.crs_json(), metadata=b.metadata())
    url = srv.url
    st, _, body = request(url, "GET", "/params", ctype=None)
    p = json.loads(body)
    assert st == 200 and p["version"] == "9.9.9" and p["entry_count"] == 3 * N + 100 and p["crs_a_vectors_count"] == 5
    st, _, body = request(url, "GET", "/crs", ctype=None)
    assert st == 200 and body == (tmp_path / "crs.json").read_bytes()
    seeds, b_rows = client.query_seeded(1000)
    want = inspire.respond_seeded_packed(crs0, edb0, inspire.SeededClientQuery(1, seeds, b_rows))
    assert want.ciphertext.b.size == 4 * N  # the crate's compat b: dimension 2 ring_dim
    st, _, body = request(url, "POST", "/query_seeded", seeded_query_body(1, seeds, b_rows, mode="tree"))
    assert st == 200, body[:300]
    ms = json.loads(body)["processing_time_ms"]
    assert body == inspire.wire.packed_response_to_json(params, want.ciphertext.a, want.ciphertext.b, ms)
    rgsw = ctx.expand_rgsw(seeds, b_rows)
    st, _, body = request(url, "POST", "/query", full_query_body(1, rgsw, mode="tree"))
    ms = json.loads(body)["processing_time_ms"]
    assert st == 200 and body == inspire.wire.packed_response_to_json(params, want.ciphertext.a, want.ciphertext.b, ms)
    srv.close()
    if impl == "native":
        py_srv.close()
    py_srv.backend.close()
    edb0.close()
    crs0.close()
