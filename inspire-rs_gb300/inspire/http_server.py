"""HTTP front end of the Respond path, with the routes, JSON shapes, status
codes and error texts of the crate's server binary (src/bin/server.rs):

    GET  /health         {"status":"ok","version":...}            (:99-104)
    GET  /params         ParamsResponse                            (:106-118)
    GET  /crs            the ServerCrs JSON                        (:238-240)
    POST /query          ClientQuery -> QueryResponse              (:120-177)
    POST /query_seeded   SeededClientQuery -> QueryResponse        (:179-236)

QueryResponse is {"response": ServerResponse, "processing_time_ms": t}
(:88-92), t measured from the start of the handler (after the body has been
deserialised, as axum runs the handler) to the end of respond.  A query in
InspiRING mode without packing keys gets 400 with {"error": "InspiRING
packing keys missing (set packing_mode=tree to use tree packing)"}; a failed
respond gets 400 with {"error": "Query processing failed: <PirError>"} (or
"Seeded query processing failed: ...").  Bodies that are not JSON get 400,
JSON of the wrong shape 422, a missing JSON content type 415, as axum's Json
extractor answers them (text bodies).

The request bodies are parsed and the replies written by the native codecs
(csrc/wire.cu); seeded InspiRING queries are answered by the GPU serving loop
(continuous batching across all connections, inspire.Server), the other
query kinds by the synchronous C-ABI calls.  Packing keys arrive in every
query (the crate serialises y_body with each query); the server keeps the
keys of recent clients resident on the GPU, keyed by the bytes of y_body, so
that a returning client's rotations are not rebuilt per query
(generate_rotations, inspiring2.rs:1309-1323, which the crate reruns for
every wire query, respond.rs:365-377).

One thread per connection (HTTP/1.1 keep-alive); the native calls release
the GIL, so parsing, responding and writing of different connections
overlap.
"""
from __future__ import annotations

import collections
import ctypes as C
import hashlib
import json
import os
import threading
import time
from http.server import BaseHTTPRequestHandler, ThreadingHTTPServer
from typing import Optional

import numpy as np

from . import _native as nat
from . import wire
from .params import InspireParams
from .pir import (ClientPackingKeys, ClientQuery, EncodedDatabase, PirError, SeededClientQuery, Server, ServerCrs,
                  _check, _ptr)

CRATE_VERSION = "0.1.2"  # env!("CARGO_PKG_VERSION") of the crate the routes mirror
KEYS_MISSING = "InspiRING packing keys missing (set packing_mode=tree to use tree packing)"


class GpuBackend:
    """The Respond calls behind the HTTP routes: one ServerCrs (device
    context), one resident EncodedDatabase, a serving loop for seeded
    InspiRING queries and a cache of resident client keys."""

    def __init__(self, crs: ServerCrs, encoded_db: EncodedDatabase, *, crs_json: Optional[bytes] = None,
                 metadata: Optional[dict] = None, max_clients: int = 4096, max_batch: int = 128,
                 max_inflight: int = 4, capacity: int = 4096):
        self.crs = crs
        self.edb = encoded_db
        self.params: InspireParams = crs.params
        self._crs_json = crs_json
        self._metadata = metadata
        self.server = Server(crs, max_batch=max_batch, max_inflight=max_inflight, capacity=capacity)
        self.max_clients = max_clients
        self._keys = collections.OrderedDict()  # digest -> [client id, queries in flight]
        self._lock = threading.Lock()

    # ---- metadata (server.rs:59-67, 106-118) ----
    def metadata(self) -> dict:
        if self._metadata is not None:
            return self._metadata
        return {"version": "1.0.0", "entry_count": int(self.edb.total_entries), "shard_count": int(self.edb.num_shards)}

    def crs_a_vectors_count(self) -> int:
        return self.crs.crs_a_vectors_count

    def crs_json(self) -> Optional[bytes]:
        return self._crs_json

    # ---- resident client keys ----
    def _acquire_client(self, y_body: np.ndarray) -> tuple:
        digest = hashlib.blake2b(np.ascontiguousarray(y_body).view(np.uint8), digest_size=16).digest()
        with self._lock:
            ent = self._keys.get(digest)
            if ent is not None:
                ent[1] += 1
                self._keys.move_to_end(digest)
                return digest, ent[0]
        cid = self._register(y_body)
        with self._lock:
            ent = self._keys.get(digest)
            if ent is not None:  # registered meanwhile by another connection
                ent[1] += 1
                self.crs.release_client(cid)
                return digest, ent[0]
            self._keys[digest] = [cid, 1]
            # evict the least recently used clients with no query in flight
            over = len(self._keys) - self.max_clients
            for d in list(self._keys):
                if over <= 0:
                    break
                c, busy = self._keys[d]
                if busy == 0:
                    del self._keys[d]
                    self.crs.release_client(c)
                    over -= 1
        return digest, cid

    def _register(self, y_body: np.ndarray) -> int:
        """Register a client's keys; when the context's device budget refuses
        them, evict idle cached clients (least recently used first) until
        they fit or nothing idle is left."""
        while True:
            try:
                return self.crs.register_client(ClientPackingKeys(y_body=y_body))
            except PirError as e:
                if e.status != nat.ERR_OUT_OF_MEMORY:
                    raise
                with self._lock:
                    idle = next((d for d, (_, busy) in self._keys.items() if busy == 0), None)
                    if idle is None:
                        raise
                    cid, _ = self._keys.pop(idle)
                self.crs.release_client(cid)

    def _release_client(self, digest: bytes) -> None:
        with self._lock:
            ent = self._keys.get(digest)
            if ent is not None:
                ent[1] -= 1

    # ---- respond ----
    def respond_seeded_inspiring(self, q: SeededClientQuery) -> np.ndarray:
        keys = q.inspiring_packing_keys
        if keys.y_body is None:  # keys present with an empty y_body: the crate's error
            from .pir import respond_seeded_inspiring

            r = respond_seeded_inspiring(self.crs, self.edb, q)
            return np.stack([r.ciphertext.a, r.ciphertext.b])
        digest, cid = self._acquire_client(keys.y_body)
        try:
            tickets, rc = self.server.submit(self.edb, [q.shard_id], q.seeds[None], q.b_rows[None], [cid])
            while rc == nat.ERR_BUSY and len(tickets) == 0:  # serving loop at capacity: wait for a slot
                time.sleep(50e-6)
                tickets, rc = self.server.submit(self.edb, [q.shard_id], q.seeds[None], q.b_rows[None], [cid])
            out = np.empty((2, self.params.plen), np.uint64)
            self.server.poll(int(tickets[0]), out)
            return out
        finally:
            self._release_client(digest)

    def respond_inspiring(self, q: ClientQuery) -> np.ndarray:
        from .pir import respond_inspiring

        r = respond_inspiring(self.crs, self.edb, q)
        return np.stack([r.ciphertext.a, r.ciphertext.b])

    def respond_seeded_packed(self, q: SeededClientQuery):
        from .pir import respond_seeded_packed

        r = respond_seeded_packed(self.crs, self.edb, q)
        return r.ciphertext.a, r.ciphertext.b

    def respond_one_packing(self, q: ClientQuery):
        from .pir import respond_one_packing

        r = respond_one_packing(self.crs, self.edb, q)
        return r.ciphertext.a, r.ciphertext.b

    def close(self):
        if self.server is not None:
            self.server.close()
            self.server = None
        with self._lock:
            for cid, _ in self._keys.values():
                try:
                    self.crs.release_client(cid)
                except PirError:
                    pass
            self._keys.clear()


def _compact(obj) -> bytes:
    return json.dumps(obj, separators=(",", ":")).encode()


def _reply_json(params: InspireParams, ct: np.ndarray, ms: int) -> bytes:
    L = nat.load()
    ct = np.ascontiguousarray(ct, dtype=np.uint64)
    cap = ct.size * 21 + 4096
    buf = C.create_string_buffer(cap)
    size = C.c_size_t(0)
    pc = params.to_c()
    _check(L.inspire_query_response_to_json(C.byref(pc), _ptr(ct), 0, None, ms, buf, cap, C.byref(size)))
    return buf.raw[:size.value]


class _Handler(BaseHTTPRequestHandler):
    protocol_version = "HTTP/1.1"
    server_version = "inspire-gb300"

    def log_message(self, fmt, *args):  # quiet, like the crate's server at INFO
        pass

    # ---- plumbing ----
    def _send(self, status: int, body: bytes, ctype: str = "application/json"):
        self.send_response(status)
        self.send_header("content-type", ctype)
        self.send_header("content-length", str(len(body)))
        self.end_headers()
        self.wfile.write(body)

    def _error(self, status: int, text: str):
        self._send(status, _compact({"error": text}))

    def _body(self) -> Optional[bytes]:
        te = self.headers.get("transfer-encoding", "")
        if "chunked" in te.lower():
            parts = []
            while True:
                size = int(self.rfile.readline().strip().split(b";")[0], 16)
                if size == 0:
                    while self.rfile.readline() not in (b"\r\n", b"\n", b""):
                        pass
                    break
                parts.append(self.rfile.read(size))
                self.rfile.readline()
            return b"".join(parts)
        n = int(self.headers.get("content-length", "0") or 0)
        if n > self.server.app.max_body:
            self._send(413, b"length limit exceeded", "text/plain; charset=utf-8")
            return None
        return self.rfile.read(n) if n else b""

    def _json_content_type(self) -> bool:
        ct = (self.headers.get("content-type") or "").split(";")[0].strip().lower()
        return ct == "application/json" or (ct.startswith("application/") and ct.endswith("+json"))

    def _rejection(self, body: bytes, err: str):
        # axum's Json extractor: 400 for a body that is not JSON, 422 for JSON
        # that does not deserialise into the target type (text bodies)
        try:
            json.loads(body)
        except ValueError as e:
            self._send(400, f"Failed to parse the request body as JSON: {e}".encode(), "text/plain; charset=utf-8")
            return
        self._send(422, f"Failed to deserialize the JSON body into the target type: {err}".encode(),
                   "text/plain; charset=utf-8")

    # ---- routes ----
    def do_GET(self):
        app = self.server.app
        path = self.path.split("?")[0]
        if path == "/health":
            self._send(200, _compact({"status": "ok", "version": CRATE_VERSION}))
        elif path == "/params":
            b = app.backend
            p, md = b.params, b.metadata()
            self._send(200, _compact({
                "version": md["version"], "ring_dim": p.ring_dim, "modulus": str(p.q), "plaintext_modulus": p.p,
                "gadget_base": p.gadget_base, "gadget_len": p.gadget_len, "entry_count": md["entry_count"],
                "shard_count": md["shard_count"], "crs_a_vectors_count": b.crs_a_vectors_count()}))
        elif path == "/crs":
            data = app.backend.crs_json()
            if data is None:
                self._error(404, "this server was started without a crs.json")
            else:
                self._send(200, data)
        else:
            self._send(404, b"", "text/plain; charset=utf-8")

    def do_POST(self):
        path = self.path.split("?")[0]
        if path not in ("/query", "/query_seeded"):
            body = self._body()
            if body is not None:
                self._send(404, b"", "text/plain; charset=utf-8")
            return
        if not self._json_content_type():
            self._body()
            self._send(415, b"Expected request with `Content-Type: application/json`", "text/plain; charset=utf-8")
            return
        body = self._body()
        if body is None:
            return
        app = self.server.app
        b = app.backend
        seeded = path == "/query_seeded"
        try:
            q = (wire.seeded_query_from_json if seeded else wire.query_from_json)(b.params, body)
        except PirError as e:
            self._rejection(body, str(e))
            return
        t0 = time.monotonic_ns()
        prefix = "Seeded query processing failed: " if seeded else "Query processing failed: "
        try:
            if q.packing_mode == "inspiring":
                if q.inspiring_packing_keys is None:
                    self._error(400, KEYS_MISSING)
                    return
                ct = b.respond_seeded_inspiring(q) if seeded else b.respond_inspiring(q)
                ms = (time.monotonic_ns() - t0) // 1_000_000
                self._send(200, _reply_json(b.params, ct, ms))
            else:
                a, bb = b.respond_seeded_packed(q) if seeded else b.respond_one_packing(q)
                ms = (time.monotonic_ns() - t0) // 1_000_000
                self._send(200, wire.packed_response_to_json(b.params, a, bb, ms))
        except PirError as e:
            self._error(400, prefix + str(e))


class PirHttpServer:
    """The crate's HTTP API (src/bin/server.rs:242-337) over a backend
    (GpuBackend by default), on `host:port` (port 0 picks a free port).
    start() serves in a background thread; close() stops it."""

    def __init__(self, backend, host: str = "127.0.0.1", port: int = 0, max_body: int = 64 << 20):
        self.backend = backend
        self.max_body = max_body
        self.httpd = ThreadingHTTPServer((host, port), _Handler)
        self.httpd.daemon_threads = True
        self.httpd.app = self
        self.thread: Optional[threading.Thread] = None

    @property
    def address(self):
        return self.httpd.server_address[:2]

    @property
    def url(self) -> str:
        h, p = self.address
        return f"http://{h}:{p}"

    def start(self) -> "PirHttpServer":
        self.thread = threading.Thread(target=self.httpd.serve_forever, kwargs={"poll_interval": 0.05}, daemon=True)
        self.thread.start()
        return self

    def serve_forever(self):
        self.httpd.serve_forever()

    def close(self):
        if self.thread is not None:
            self.httpd.shutdown()
            self.thread.join()
            self.thread = None
        self.httpd.server_close()

    @classmethod
    def from_data_dir(cls, data_dir: str, params: Optional[InspireParams] = None, mode: str = "crt_fixed",
                      device: int = 0, mmap: bool = False, host: str = "0.0.0.0", port: int = 3000,
                      **backend_kw) -> "PirHttpServer":
        """Start-up of the crate's server (server.rs:242-305): crs.json, then
        encoded_db.json or (mmap) the binary shards under shards/, and
        metadata.json when present, all from data_dir; the database is made
        resident in HBM either way."""
        params = params or InspireParams()
        with open(os.path.join(data_dir, "crs.json"), "rb") as f:
            crs_json = f.read()
        crs = ServerCrs.load_json(params, crs_json, mode=mode, device=device)
        if mmap:
            shards = os.path.join(data_dir, "shards")
            if not os.path.isdir(shards):
                raise FileNotFoundError(f"Shards directory not found: {shards}. Run setup with --binary-output first.")
            edb = EncodedDatabase.load_shards(crs, shards)
        else:
            edb = EncodedDatabase.load_json(crs, os.path.join(data_dir, "encoded_db.json"))
        meta_path = os.path.join(data_dir, "metadata.json")
        metadata = None
        if os.path.exists(meta_path):
            with open(meta_path) as f:
                m = json.load(f)
            metadata = {"version": m["version"], "entry_count": int(m["entry_count"]),
                        "shard_count": int(m["shard_count"])}
        else:
            metadata = {"version": "1.0.0", "entry_count": 0, "shard_count": 0}
        backend = GpuBackend(crs, edb, crs_json=crs_json, metadata=metadata, **backend_kw)
        return cls(backend, host, port)


class NativeHttpServer:
    """The same routes served by the library itself (csrc/http.cu,
    inspire_http_start): C++ threads per connection, no interpreter on the
    request path.  Seeded InspiRING queries go through a serving loop on
    the context (one is created unless `server` is given); client keys are
    cached as GpuBackend caches them.  Same interface as PirHttpServer."""

    def __init__(self, crs: ServerCrs, encoded_db: EncodedDatabase, host: str = "127.0.0.1", port: int = 0, *,
                 server: Optional[Server] = None, crs_json: Optional[bytes] = None, metadata: Optional[dict] = None,
                 max_clients: int = 4096, max_body: int = 64 << 20, max_batch: int = 128, max_inflight: int = 4,
                 capacity: int = 4096):
        self.L = nat.load()
        self.crs, self.edb = crs, encoded_db
        self._own_server = server is None
        self.server = server if server is not None else Server(crs, max_batch=max_batch, max_inflight=max_inflight,
                                                               capacity=capacity)
        md = metadata or {"version": "1.0.0", "entry_count": int(encoded_db.total_entries),
                          "shard_count": int(encoded_db.num_shards)}
        cfg = nat.HttpConfigC()
        self.L.inspire_http_config_default(C.byref(cfg))
        self._host = host.encode()
        self._version = str(md["version"]).encode()
        cfg.host, cfg.port, cfg.max_clients, cfg.max_body = self._host, port, max_clients, max_body
        cfg.version, cfg.entry_count, cfg.shard_count = self._version, int(md["entry_count"]), int(md["shard_count"])
        h = C.c_void_p()
        data = crs_json or b""
        _check(self.L.inspire_http_start(crs.h, encoded_db.h, self.server.h, C.byref(cfg), data, len(data), C.byref(h)))
        self.h = h

    @property
    def address(self):
        return self._host.decode(), int(self.L.inspire_http_port(self.h))

    @property
    def url(self) -> str:
        h, p = self.address
        return f"http://{h}:{p}"

    def start(self) -> "NativeHttpServer":
        return self  # accepting since construction

    def close(self):
        if getattr(self, "h", None):
            self.L.inspire_http_stop(self.h)
            self.h = None
        if self._own_server and self.server is not None:
            self.server.close()
            self.server = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def main(argv=None):
    """inspire-server's command line (server.rs:30-46): --data-dir, --bind,
    --mmap; plus --mode and --device of the GPU build."""
    import argparse

    ap = argparse.ArgumentParser(description="InsPIRe PIR server (GB300)")
    ap.add_argument("--data-dir", default="inspire_data")
    ap.add_argument("--bind", default="0.0.0.0:3000")
    ap.add_argument("--mmap", action="store_true")
    ap.add_argument("--mode", default="crt_fixed", choices=["crt_fixed", "compat"])
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--python", action="store_true", help="serve from Python (http.server) instead of the library")
    a = ap.parse_args(argv)
    host, port = a.bind.rsplit(":", 1)
    srv = PirHttpServer.from_data_dir(a.data_dir, mode=a.mode, device=a.device, mmap=a.mmap, host=host,
                                      port=0 if not a.python else int(port))
    if a.python:
        print(f"Listening on: {srv.url}", flush=True)
        try:
            srv.serve_forever()
        finally:
            srv.backend.close()
        return
    b = srv.backend
    srv.close()
    native = NativeHttpServer(b.crs, b.edb, host, int(port), server=b.server, crs_json=b.crs_json(),
                              metadata=b.metadata())
    print(f"Listening on: {native.url}", flush=True)
    try:
        while True:
            time.sleep(3600)
    finally:
        native.close()
        b.close()


if __name__ == "__main__":
    main()
