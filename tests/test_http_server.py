"""The HTTP front end (inspire/http_server.py) on CPU: routes, JSON shapes,
status codes and error texts of the crate's server (src/bin/server.rs:88-236,
311-317), tested the way tests/http_inspiring.rs:80-168 tests it -- an
in-process server on 127.0.0.1:0, real requests -- over a backend that
answers with the oracle (test infrastructure), so that the request parsing
and reply writing run on real query bytes without a GPU."""
import http.client
import json

import numpy as np
import pytest

from http_helpers import N, ciphertext_of, full_query_body, request, seeded_query_body

ENTRY = 32
W_SEED = bytes(range(33, 65))


class OracleBackend:
    """Answers as the crate's respond functions do, through the oracle."""

    def __init__(self, O, inspire, db, n_shards):
        self.O = O
        self.ctx = O.Ctx()
        self.pack = O.Pack(self.ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
        self.params = inspire.InspireParams(p=1 << 16)
        self.db = db
        self.n_shards = n_shards
        self.PirError = inspire.PirError

    def metadata(self):
        return {"version": "1.0.0", "entry_count": self.db.size // ENTRY, "shard_count": self.n_shards}

    def crs_a_vectors_count(self):
        return 2048

    def crs_json(self):
        return b'{"inspiring_num_columns":16}'

    def _respond(self, shard_id, rgsw, keys):
        if shard_id >= self.n_shards:
            raise self.PirError(f"Shard {shard_id} not found")
        if keys.y_body is None:
            raise self.PirError("InspiRING packing keys invalid: y_all and y_body are both empty")
        shard = self.ctx.encode_shard(self.db, ENTRY, shard_id)
        return self.ctx.respond_inspiring(shard, rgsw, W_SEED, mode=self.O.MODE_CRT_FIXED, pack=self.pack,
                                          y_body=keys.y_body)

    def respond_seeded_inspiring(self, q):
        return self._respond(q.shard_id, self.ctx.expand_rgsw(q.seeds, q.b_rows), q.inspiring_packing_keys)

    def respond_inspiring(self, q):
        return self._respond(q.shard_id, q.rgsw.reshape(12, -1), q.inspiring_packing_keys)

    def respond_seeded_packed(self, q):
        raise self.PirError("tree packing is not served by this backend")

    respond_one_packing = respond_seeded_packed


@pytest.fixture(scope="module")
def served(oracle_mod):
    import build_lib

    build_lib.build()
    import inspire
    from inspire.http_server import PirHttpServer

    rng = np.random.default_rng(31)
    db = rng.integers(0, 256, size=(N + 500) * ENTRY, dtype=np.uint8)
    backend = OracleBackend(oracle_mod, inspire, db, 2)
    srv = PirHttpServer(backend, "127.0.0.1", 0).start()
    client = oracle_mod.Client(backend.ctx, seed=4, rng_seed=44)
    y_body, _ = client.packing_keys(backend.pack)
    yield dict(srv=srv, url=srv.url, backend=backend, client=client, y_body=y_body, db=db, inspire=inspire)
    srv.close()


def test_health_params_crs(served):
    url = served["url"]
    st, ct, body = request(url, "GET", "/health", ctype=None)
    assert st == 200 and ct == "application/json" and body == b'{"status":"ok","version":"0.1.2"}'
    st, ct, body = request(url, "GET", "/params", ctype=None)
    assert st == 200
    assert json.loads(body) == {"version": "1.0.0", "ring_dim": 2048, "modulus": str(268369921 * 249561089),
                                "plaintext_modulus": 65536, "gadget_base": 1 << 20, "gadget_len": 3,
                                "entry_count": N + 500, "shard_count": 2, "crs_a_vectors_count": 2048}
    assert list(json.loads(body)) == ["version", "ring_dim", "modulus", "plaintext_modulus", "gadget_base",
                                      "gadget_len", "entry_count", "shard_count", "crs_a_vectors_count"]
    st, _, body = request(url, "GET", "/crs", ctype=None)
    assert st == 200 and body == b'{"inspiring_num_columns":16}'
    st, _, _ = request(url, "GET", "/nowhere", ctype=None)
    assert st == 404


def test_seeded_and_full_queries(served):
    """Success path over one keep-alive connection: the reply is the oracle's
    response in the crate's QueryResponse shape, and extracts to the entry."""
    W = served
    be, client = W["backend"], W["client"]
    host, port = W["srv"].address
    conn = http.client.HTTPConnection(host, port, timeout=120)
    for idx in (5, N + 77):
        sid, local = divmod(idx, N)
        seeds, b_rows = client.query_seeded(local)
        want = be.ctx.respond_inspiring(be.ctx.encode_shard(W["db"], ENTRY, sid), be.ctx.expand_rgsw(seeds, b_rows),
                                        W_SEED, mode=be.O.MODE_CRT_FIXED, pack=be.pack, y_body=W["y_body"])
        st, ct, body = request(conn, "POST", "/query_seeded", seeded_query_body(sid, seeds, b_rows, W["y_body"]))
        assert st == 200 and ct == "application/json", body[:200]
        obj = json.loads(body)
        assert list(obj) == ["response", "processing_time_ms"]
        assert obj["response"]["column_ciphertexts"] == []
        got = ciphertext_of(body)
        assert np.array_equal(got, want)
        # the reply is exactly the native writer's bytes for that response
        ms = obj["processing_time_ms"]
        resp = W["inspire"].ServerResponse(W["inspire"].RlweCiphertext(want[0], want[1]), [])
        assert body == W["inspire"].wire.query_response_to_json(be.params, resp, ms)
        assert np.array_equal(client.extract_inspiring(got, ENTRY), W["db"][idx * ENTRY:(idx + 1) * ENTRY])
        rgsw = be.ctx.expand_rgsw(seeds, b_rows)
        st, _, body = request(conn, "POST", "/query", full_query_body(sid, rgsw, W["y_body"]))
        assert st == 200 and np.array_equal(ciphertext_of(body), want)
    conn.close()


def test_errors_follow_the_crate(served):
    W = served
    url, client = W["url"], W["client"]
    seeds, b_rows = client.query_seeded(9)
    # InspiRING without packing keys (server.rs:131-140, 186-195)
    for path, body in (("/query_seeded", seeded_query_body(0, seeds, b_rows)),
                       ("/query", full_query_body(0, W["backend"].ctx.expand_rgsw(seeds, b_rows)))):
        st, ct, reply = request(url, "POST", path, body)
        assert st == 400 and ct == "application/json"
        assert json.loads(reply) == {"error": "InspiRING packing keys missing (set packing_mode=tree to use tree "
                                              "packing)"}
    # respond errors, prefixed as server.rs:162-169 / 220-227 do
    st, _, reply = request(url, "POST", "/query_seeded", seeded_query_body(7, seeds, b_rows, W["y_body"]))
    assert st == 400 and json.loads(reply) == {"error": "Seeded query processing failed: Shard 7 not found"}
    st, _, reply = request(url, "POST", "/query", full_query_body(9, W["backend"].ctx.expand_rgsw(seeds, b_rows),
                                                                  W["y_body"]))
    assert st == 400 and json.loads(reply) == {"error": "Query processing failed: Shard 9 not found"}
    empty = json.loads(seeded_query_body(0, seeds, b_rows, W["y_body"]))
    empty["inspiring_packing_keys"]["y_body"] = []
    st, _, reply = request(url, "POST", "/query_seeded", json.dumps(empty).encode())
    assert st == 400
    assert json.loads(reply)["error"] == ("Seeded query processing failed: InspiRING packing keys invalid: y_all "
                                          "and y_body are both empty")
    # extractor rejections: not JSON (400), wrong shape (422), wrong content type (415)
    st, ct, reply = request(url, "POST", "/query_seeded", b'{"shard_id": 1,')
    assert st == 400 and ct.startswith("text/plain") and reply.startswith(b"Failed to parse the request body")
    st, _, reply = request(url, "POST", "/query_seeded", b'{"shard_id": 1}')
    assert st == 422 and reply.startswith(b"Failed to deserialize the JSON body")
    st, _, reply = request(url, "POST", "/query_seeded", seeded_query_body(0, seeds, b_rows, W["y_body"]),
                           ctype="text/plain")
    assert st == 415
    st, _, _ = request(url, "POST", "/query_seeded", b'{"shard_id": 007}')
    assert st == 400  # serde_json rejects leading zeros: not JSON


def test_load_generator_closed_and_open_loop(served):
    """inspire.http_load against the in-process server: spawned client
    processes, keep-alive connections, every reply 200."""
    from inspire import http_load

    W = served
    seeds, b_rows = W["client"].query_seeded(11)
    body = http_load.seeded_query_json(0, seeds, b_rows, W["y_body"])
    assert body == seeded_query_body(0, seeds, b_rows, W["y_body"])  # the same bytes as serde_json's
    r = http_load.run_load(W["url"], [body], 2, duration_s=0.6, warmup_s=0.1)
    assert r["errors"] == 0 and r["requests"] >= 1 and r["p50_ms"] > 0
    r = http_load.run_load(W["url"], [body], 2, duration_s=0.6, warmup_s=0.1, rate=4.0)
    assert r["errors"] == 0 and r["offered_rps"] == 4.0
