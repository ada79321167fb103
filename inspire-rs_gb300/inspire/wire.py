"""Wire formats of the crate's HTTP API through the native codecs
(include/inspire_gpu.h, csrc/wire.cu): the SeededClientQuery JSON request,
the server's JSON reply and ServerResponse's bincode form."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .params import InspireParams
from .pir import ClientPackingKeys, ClientQuery, PirError, SeededClientQuery, ServerResponse, _check, _ptr


def seeded_query_from_json(params: InspireParams, body: bytes | str) -> SeededClientQuery:
    """Parse a SeededClientQuery JSON body (pir/query.rs:138-150)."""
    L = nat.load()
    raw = body.encode() if isinstance(body, str) else bytes(body)
    ell, plen = params.gadget_len, params.plen
    seeds = np.zeros((2 * ell, 32), np.uint8)
    b_rows = np.zeros((2 * ell, plen), np.uint64)
    y_body = np.zeros((ell, plen), np.uint64)
    sid, mode, keys = C.c_uint32(0), C.c_int32(0), C.c_int32(0)
    pc = params.to_c()
    _check(L.inspire_seeded_query_from_json(C.byref(pc), raw, len(raw), C.byref(sid), _ptr(seeds), _ptr(b_rows),
                                            C.byref(mode), C.byref(keys), _ptr(y_body)))
    return SeededClientQuery(int(sid.value), seeds, b_rows, "tree" if mode.value else "inspiring",
                             _keys(keys.value, y_body))


def _keys(flag: int, y_body: np.ndarray):
    # 0: no inspiring_packing_keys; 1: with y_body; 2: present with an empty
    # y_body (respond reports the keys invalid, as the crate does)
    return None if flag == 0 else ClientPackingKeys(y_body=y_body if flag == 1 else None)


def query_from_json(params: InspireParams, body: bytes | str) -> ClientQuery:
    """Parse a ClientQuery JSON body (pir/query.rs:119-132), the /query
    request of the crate's server."""
    L = nat.load()
    raw = body.encode() if isinstance(body, str) else bytes(body)
    ell, plen = params.gadget_len, params.plen
    rgsw = np.zeros((2 * ell, 2, plen), np.uint64)
    y_body = np.zeros((ell, plen), np.uint64)
    sid, mode, keys = C.c_uint32(0), C.c_int32(0), C.c_int32(0)
    pc = params.to_c()
    _check(L.inspire_query_from_json(C.byref(pc), raw, len(raw), C.byref(sid), _ptr(rgsw), C.byref(mode),
                                     C.byref(keys), _ptr(y_body)))
    return ClientQuery(int(sid.value), rgsw, "tree" if mode.value else "inspiring", _keys(keys.value, y_body))


def packed_response_to_json(params: InspireParams, a: np.ndarray, b: np.ndarray, processing_time_ms: int = 0) -> bytes:
    """The server's JSON reply for a tree-packing response (b may have the
    crate's compat dimension 2 ring_dim)."""
    L = nat.load()
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    pc = params.to_c()
    size = C.c_size_t(0)
    cap = (a.size + b.size) * 21 + 4096
    buf = C.create_string_buffer(cap)
    _check(L.inspire_packed_response_to_json(C.byref(pc), _ptr(a), _ptr(b), b.size, processing_time_ms, buf, cap,
                                             C.byref(size)))
    return buf.raw[:size.value]


def _ct_arrays(response: ServerResponse):
    ct = np.ascontiguousarray(np.concatenate([response.ciphertext.a, response.ciphertext.b]), dtype=np.uint64)
    cols = None
    if response.column_ciphertexts:
        cols = np.ascontiguousarray(np.stack([np.concatenate([c.a, c.b]) for c in response.column_ciphertexts]),
                                    dtype=np.uint64)
    return ct, cols


def query_response_to_json(params: InspireParams, response: ServerResponse, processing_time_ms: int = 0) -> bytes:
    """The server's JSON reply {"response": ..., "processing_time_ms": t}
    (src/bin/server.rs:88-92)."""
    L = nat.load()
    ct, cols = _ct_arrays(response)
    n = 0 if cols is None else cols.shape[0]
    pc = params.to_c()
    size = C.c_size_t(0)
    # upper bound: every number at most 20 digits plus a separator
    cap = (2 + 2 * n) * params.plen * 21 + 4096
    buf = C.create_string_buffer(cap)
    _check(L.inspire_query_response_to_json(C.byref(pc), _ptr(ct), n, _ptr(cols), processing_time_ms, buf, cap,
                                            C.byref(size)))
    return buf.raw[:size.value]


def server_response_to_bincode(params: InspireParams, response: ServerResponse) -> bytes:
    """ServerResponse::to_binary (pir/respond.rs:43-50)."""
    L = nat.load()
    ct, cols = _ct_arrays(response)
    n = 0 if cols is None else cols.shape[0]
    pc = params.to_c()
    size = C.c_size_t(0)
    cap = (2 + 2 * n) * (8 * params.plen + 64) + 8
    buf = (C.c_uint8 * cap)()
    _check(L.inspire_server_response_to_bincode(C.byref(pc), _ptr(ct), n, _ptr(cols), buf, cap, C.byref(size)))
    return bytes(buf)[:size.value]


__all__ = ["seeded_query_from_json", "query_from_json", "query_response_to_json", "packed_response_to_json",
           "server_response_to_bincode", "PirError"]
