"""Server Respond API of the InsPIRe PIR protocol on one GB300.

Mirrors the Respond surface of the Rust crate igor53627/inspire-rs v0.1.2
(src/pir/mod.rs:57-71): `respond_seeded_inspiring`, `respond_inspiring`,
`respond_seeded_with_variant`, the query/response types and `PirError`, with
the same argument meaning and error texts.  Every call goes through the C ABI
of include/inspire_gpu.h; responses are computed by the CUDA kernels.

Polynomials are numpy uint64 arrays of shape (crt_count * ring_dim,), residue
major, canonical: the layout of the crate's `Poly::coeffs` (poly.rs:64-77).
"""
from __future__ import annotations

import atexit
import ctypes as C
import weakref
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _native as nat
from .params import InspireParams, InspireVariant


# Live native handles, closed databases-first at interpreter exit (before the
# CUDA runtime tears down) whatever order the garbage collector would pick.
_LIVE_DBS: "weakref.WeakSet" = weakref.WeakSet()
_LIVE_CRS: "weakref.WeakSet" = weakref.WeakSet()
_LIVE_SERVERS: "weakref.WeakSet" = weakref.WeakSet()
_LIVE_PINNED: "weakref.WeakSet" = weakref.WeakSet()


@atexit.register
def _close_all() -> None:
    for srv in list(_LIVE_SERVERS):
        srv.close()
    for buf in list(_LIVE_PINNED):
        buf.close()
    for db in list(_LIVE_DBS):
        db.close()
    for crs in list(_LIVE_CRS):
        crs.close()


class PirError(Exception):
    """PirError(String) of src/pir/error.rs:13 (plus the native status code)."""

    def __init__(self, message: str, status: int = 0):
        super().__init__(message)
        self.status = status


def _check(rc: int) -> None:
    if rc != nat.OK:
        raise PirError(nat.last_error(), rc)


def _u64(a, shape=None) -> np.ndarray:
    arr = np.ascontiguousarray(a, dtype=np.uint64)
    if shape is not None and arr.shape != shape:
        arr = arr.reshape(shape)
    return arr


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@dataclass
class ClientPackingKeys:
    """ClientPackingKeys (inspiring2.rs:604-628): y_body (gadget_len polys)
    and/or the in-process y_all ((num_columns-1)*gadget_len polys)."""

    y_body: Optional[np.ndarray] = None
    y_all: Optional[np.ndarray] = None


@dataclass
class SeededClientQuery:
    """SeededClientQuery (query.rs:138-150): seeds (2*ell, 32) uint8 and
    b_rows (2*ell, crt*n) uint64 of the SeededRgswCiphertext."""

    shard_id: int
    seeds: np.ndarray
    b_rows: np.ndarray
    packing_mode: str = "inspiring"
    inspiring_packing_keys: Optional[ClientPackingKeys] = None


@dataclass
class ClientQuery:
    """ClientQuery (query.rs:119-132): rgsw = (2*ell, 2, crt*n) rows (a, b)."""

    shard_id: int
    rgsw: np.ndarray
    packing_mode: str = "inspiring"
    inspiring_packing_keys: Optional[ClientPackingKeys] = None


@dataclass
class RlweCiphertext:
    a: np.ndarray
    b: np.ndarray


@dataclass
class ServerResponse:
    """ServerResponse (respond.rs:31-37)."""

    ciphertext: RlweCiphertext
    column_ciphertexts: list = field(default_factory=list)


class ServerCrs:
    """The InspiRING part of ServerCrs (setup.rs:52-87) bound to one GPU.

    Holds the device context (NTT tables, constants) and the rotated w_mask
    table built once from `inspiring_w_seed` for `inspiring_num_columns`.
    `mode` selects the NTT-domain automorphism semantics: "compat" reproduces
    the crate bit for bit; "crt_fixed" applies the permutation to both CRT
    residues (the responses decrypt)."""

    def __init__(self, params: InspireParams, inspiring_w_seed: bytes, inspiring_num_columns: int,
                 mode: str = "crt_fixed", device: int = 0, _crs_json: Optional[bytes] = None):
        self.L = nat.load()
        self.params = params
        self.mode = mode
        if mode not in ("compat", "crt_fixed"):
            raise ValueError("mode must be 'compat' or 'crt_fixed'")
        pc = params.to_c()
        h = C.c_void_p()
        _check(self.L.inspire_ctx_create(C.byref(pc), device, nat.MODE_COMPAT if mode == "compat" else nat.MODE_CRT_FIXED,
                                         C.byref(h)))
        self.h = h
        _LIVE_CRS.add(self)
        if _crs_json is not None:
            _check(self.L.inspire_crs_load_json(self.h, _crs_json, len(_crs_json)))
            seed = (C.c_uint8 * 32)()
            cols, galois = C.c_uint32(0), C.c_int32(0)
            _check(self.L.inspire_crs_info(self.h, C.cast(seed, C.c_void_p), C.byref(cols), C.byref(galois)))
            inspiring_w_seed, inspiring_num_columns = bytes(seed), cols.value
        self.inspiring_w_seed = bytes(inspiring_w_seed)
        self.inspiring_num_columns = int(inspiring_num_columns)
        if _crs_json is None:
            seed = (C.c_uint8 * 32).from_buffer_copy(self.inspiring_w_seed)
            _check(self.L.inspire_crs_load(self.h, C.cast(seed, C.c_void_p), self.inspiring_num_columns))

    @classmethod
    def load_json(cls, params: InspireParams, crs_json, mode: str = "crt_fixed", device: int = 0) -> "ServerCrs":
        """The server's crs.json (serde_json of ServerCrs, setup.rs:52-87) --
        a path or the JSON bytes: the InspiRING seed and column count, and
        the Galois keys if present; params must match."""
        data = crs_json
        if isinstance(data, str):
            with open(data, "rb") as f:
                data = f.read()
        return cls(params, b"", 0, mode=mode, device=device, _crs_json=bytes(data))

    def close(self):
        if getattr(self, "h", None):
            for db in list(_LIVE_DBS):
                if db.crs is self:
                    db.close()
            self.L.inspire_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ring_dim(self) -> int:
        return self.params.ring_dim

    def modulus(self) -> int:
        return self.params.q

    # ---- client key residency (serving) ----
    def register_client(self, keys: ClientPackingKeys) -> int:
        yb = None if keys.y_body is None else _u64(keys.y_body)
        ya = None if keys.y_all is None else _u64(keys.y_all)
        cid = C.c_int32()
        _check(self.L.inspire_client_register(self.h, _ptr(yb), _ptr(ya), C.byref(cid)))
        return cid.value

    def release_client(self, client_id: int) -> None:
        _check(self.L.inspire_client_release(self.h, client_id))

    def set_device_budget(self, nbytes: int) -> None:
        """Admission by device memory: every device buffer of this context
        (tables, databases, client keys, serving slots, staging) counts
        against `nbytes` (0: no limit); what would exceed it is refused with
        PirError (status ERR_OUT_OF_MEMORY) before allocating."""
        _check(self.L.inspire_ctx_set_device_budget(self.h, int(nbytes)))

    @property
    def pair_threshold(self) -> int:
        """Launches of at most this many queries run each query on a cluster
        of two CTAs, one per CRT residue (lower latency); larger ones on one
        CTA per query.  Default: half the SM count; 0 disables the cluster
        kernel.  Responses are identical either way."""
        return int(self.L.inspire_ctx_pair_threshold(self.h))

    @pair_threshold.setter
    def pair_threshold(self, max_queries: int) -> None:
        _check(self.L.inspire_ctx_set_pair_threshold(self.h, int(max_queries)))

    def device_memory(self):
        """(bytes in use, budget) of this context's device memory."""
        used, budget = C.c_uint64(0), C.c_uint64(0)
        _check(self.L.inspire_ctx_device_memory(self.h, C.byref(used), C.byref(budget)))
        return int(used.value), int(budget.value)

    @property
    def crs_a_vectors_count(self) -> int:
        """crs_a_vectors in the loaded crs.json (0 if not loaded from one)."""
        return int(self.L.inspire_crs_a_vectors_count(self.h))

    def inspiring_precomp(self, a_polys: np.ndarray):
        """setup's inspiring_precomp (setup.rs:194-224): packing_offline
        (inspiring2.rs:926-1041) over num_columns a-polys (coefficient form,
        shape (num_columns, plen)) on the GPU.  Returns (a_hat (plen,),
        bold_t ((num_columns-1)*gadget_len, plen)), coefficient form."""
        g, ell, plen = self.inspiring_num_columns, self.params.gadget_len, self.params.plen
        a = _u64(a_polys).reshape(g, plen)
        a_hat = np.zeros(plen, np.uint64)
        bold_t = np.zeros((max(1, (g - 1) * ell), plen), np.uint64)
        _check(self.L.inspire_inspiring_precomp(self.h, _ptr(a), _ptr(a_hat), _ptr(bold_t)))
        return a_hat, bold_t[:(g - 1) * ell]

    def load_galois_keys(self, galois_keys: np.ndarray) -> None:
        """ServerCrs.galois_keys (setup.rs:164-173) for tree packing: log2(d)
        key-switching matrices of 2*gadget_len rows [a, b] each, shape
        (log2 d, 2*ell, plen), uint64 residues."""
        keys = _u64(galois_keys)
        _check(self.L.inspire_crs_load_galois_keys(self.h, _ptr(keys), keys.shape[0]))


class EncodedDatabase:
    """EncodedDatabase (setup.rs:104-120) resident in HBM: shards of ring_dim
    entries, 16-bit columns (encode_db.rs:106-181), plus the contracted form
    the Respond kernel reads."""

    def __init__(self, crs: ServerCrs, database: bytes | np.ndarray, entry_size: int, _handle=None):
        self.crs = crs
        self.L = crs.L
        self.entry_size = int(entry_size)
        if _handle is not None:
            self.h = _handle
            self.total_entries = self.num_shards * crs.params.ring_dim
            _LIVE_DBS.add(self)
            return
        raw = np.frombuffer(database, dtype=np.uint8) if isinstance(database, (bytes, bytearray)) else \
            np.ascontiguousarray(database, dtype=np.uint8).reshape(-1)
        self.total_entries = raw.size // self.entry_size if self.entry_size else 0
        h = C.c_void_p()
        _check(self.L.inspire_db_create(crs.h, raw.ctypes.data_as(C.c_void_p), self.total_entries, self.entry_size,
                                        C.byref(h)))
        self.h = h
        _LIVE_DBS.add(self)

    @classmethod
    def load_shards(cls, crs: ServerCrs, directory: str) -> "EncodedDatabase":
        """Load the crate's binary shard files (save_shards_binary,
        mmap.rs:19-53) from `directory` straight into HBM."""
        h = C.c_void_p()
        _check(crs.L.inspire_db_load_shards(crs.h, str(directory).encode(), C.byref(h)))
        return cls(crs, b"", 2 * crs.inspiring_num_columns, _handle=h)

    @classmethod
    def load_json(cls, crs: ServerCrs, encoded_db_json) -> "EncodedDatabase":
        """Load the server's encoded_db.json (serde_json of EncodedDatabase,
        server.rs:292-301) -- a path or the JSON bytes -- into HBM."""
        data = encoded_db_json
        if isinstance(data, str):
            with open(data, "rb") as f:
                data = f.read()
        data = bytes(data)
        h = C.c_void_p()
        _check(crs.L.inspire_db_load_json(crs.h, data, len(data), C.byref(h)))
        return cls(crs, b"", 2 * crs.inspiring_num_columns, _handle=h)

    def save_shards(self, directory: str) -> None:
        """Write this database as the crate's binary shard files."""
        pc = self.crs.params.to_c()
        _check(self.L.inspire_db_save_shards(self.h, C.byref(pc), str(directory).encode()))

    @property
    def num_shards(self) -> int:
        return int(self.L.inspire_db_num_shards(self.h))

    @property
    def device_bytes(self) -> int:
        return int(self.L.inspire_db_device_bytes(self.h))

    def index_to_shard(self, global_idx: int):
        """ShardConfig::index_to_shard (params.rs:553-558)."""
        n = self.crs.params.ring_dim
        return global_idx // n, global_idx % n

    def close(self):
        if getattr(self, "h", None):
            self.L.inspire_db_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _response(out: np.ndarray, plen: int) -> ServerResponse:
    return ServerResponse(RlweCiphertext(out[:plen].copy(), out[plen:].copy()), [])


def respond_seeded_inspiring(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededClientQuery) -> ServerResponse:
    """respond_seeded_inspiring (respond.rs:391-398)."""
    plen = crs.params.plen
    ell = crs.params.gadget_len
    seeds = np.ascontiguousarray(query.seeds, dtype=np.uint8).reshape(2 * ell, 32)
    b_rows = _u64(query.b_rows).reshape(2 * ell, plen)
    keys = query.inspiring_packing_keys
    yb = None if keys is None or keys.y_body is None else _u64(keys.y_body)
    ya = None if keys is None or keys.y_all is None else _u64(keys.y_all)
    q = nat.SeededQueryC(query.shard_id, seeds.ctypes.data_as(C.c_void_p), b_rows.ctypes.data_as(C.c_void_p),
                         1 if keys is not None else 0, _ptr(yb), _ptr(ya))
    out = np.zeros(2 * plen, dtype=np.uint64)
    _check(crs.L.inspire_respond_seeded_inspiring(crs.h, encoded_db.h, C.byref(q), _ptr(out)))
    return _response(out, plen)


def respond_inspiring(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery) -> ServerResponse:
    """respond_inspiring (respond.rs:284-386)."""
    plen = crs.params.plen
    ell = crs.params.gadget_len
    rgsw = _u64(query.rgsw).reshape(2 * ell, 2, plen)
    keys = query.inspiring_packing_keys
    yb = None if keys is None or keys.y_body is None else _u64(keys.y_body)
    ya = None if keys is None or keys.y_all is None else _u64(keys.y_all)
    q = nat.QueryC(query.shard_id, rgsw.ctypes.data_as(C.c_void_p), 1 if keys is not None else 0, _ptr(yb), _ptr(ya))
    out = np.zeros(2 * plen, dtype=np.uint64)
    _check(crs.L.inspire_respond_inspiring(crs.h, encoded_db.h, C.byref(q), _ptr(out)))
    return _response(out, plen)


def _nopacking_response(out: np.ndarray, cols: Optional[np.ndarray], plen: int) -> ServerResponse:
    columns = [] if cols is None else [RlweCiphertext(c[0].copy(), c[1].copy()) for c in cols]
    return ServerResponse(RlweCiphertext(out[:plen].copy(), out[plen:].copy()), columns)


def respond(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery,
            with_columns: bool = True) -> ServerResponse:
    """respond (respond.rs:71-115), the NoPacking variant: column_ciphertexts
    holds one RLWE ciphertext per shard column (skipped when with_columns is
    False), ciphertext their sum."""
    plen = crs.params.plen
    ell = crs.params.gadget_len
    rgsw = _u64(query.rgsw).reshape(2 * ell, 2, plen)
    q = nat.QueryC(query.shard_id, rgsw.ctypes.data_as(C.c_void_p), 0, None, None)
    out = np.zeros(2 * plen, dtype=np.uint64)
    cols = np.zeros((crs.inspiring_num_columns, 2, plen), dtype=np.uint64) if with_columns else None
    _check(crs.L.inspire_respond(crs.h, encoded_db.h, C.byref(q), _ptr(out), _ptr(cols)))
    return _nopacking_response(out, cols, plen)


def respond_seeded(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededClientQuery,
                   with_columns: bool = True) -> ServerResponse:
    """respond_seeded (respond.rs:408-415): expand, then NoPacking respond."""
    plen = crs.params.plen
    ell = crs.params.gadget_len
    seeds = np.ascontiguousarray(query.seeds, dtype=np.uint8).reshape(2 * ell, 32)
    b_rows = _u64(query.b_rows).reshape(2 * ell, plen)
    q = nat.SeededQueryC(query.shard_id, seeds.ctypes.data_as(C.c_void_p), b_rows.ctypes.data_as(C.c_void_p),
                         0, None, None)
    out = np.zeros(2 * plen, dtype=np.uint64)
    cols = np.zeros((crs.inspiring_num_columns, 2, plen), dtype=np.uint64) if with_columns else None
    _check(crs.L.inspire_respond_seeded(crs.h, encoded_db.h, C.byref(q), _ptr(out), _ptr(cols)))
    return _nopacking_response(out, cols, plen)


def _packed_response(out_a, out_b, words) -> ServerResponse:
    return ServerResponse(RlweCiphertext(out_a, out_b[:words]), [])


def respond_one_packing(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery) -> ServerResponse:
    """respond_one_packing (respond.rs:213-268): column products, then
    pack_lwes with the CRS's Galois keys (load_galois_keys).  In compat mode
    with more than one column the b polynomial has 2*plen words, as the
    crate's pack_lwes returns it (automorph_pack.rs:474-484)."""
    plen = crs.params.plen
    ell = crs.params.gadget_len
    rgsw = _u64(query.rgsw).reshape(2 * ell, 2, plen)
    q = nat.QueryC(query.shard_id, rgsw.ctypes.data_as(C.c_void_p), 0, None, None)
    out_a = np.zeros(plen, dtype=np.uint64)
    out_b = np.zeros(2 * plen, dtype=np.uint64)
    words = C.c_uint32(0)
    _check(crs.L.inspire_respond_one_packing(crs.h, encoded_db.h, C.byref(q), _ptr(out_a), _ptr(out_b),
                                             C.byref(words)))
    return _packed_response(out_a, out_b, words.value)


def respond_seeded_packed(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededClientQuery) -> ServerResponse:
    """respond_seeded_packed (respond.rs:428-435): expand, then
    respond_one_packing."""
    plen = crs.params.plen
    ell = crs.params.gadget_len
    seeds = np.ascontiguousarray(query.seeds, dtype=np.uint8).reshape(2 * ell, 32)
    b_rows = _u64(query.b_rows).reshape(2 * ell, plen)
    q = nat.SeededQueryC(query.shard_id, seeds.ctypes.data_as(C.c_void_p), b_rows.ctypes.data_as(C.c_void_p),
                         0, None, None)
    out_a = np.zeros(plen, dtype=np.uint64)
    out_b = np.zeros(2 * plen, dtype=np.uint64)
    words = C.c_uint32(0)
    _check(crs.L.inspire_respond_seeded_packed(crs.h, encoded_db.h, C.byref(q), _ptr(out_a), _ptr(out_b),
                                               C.byref(words)))
    return _packed_response(out_a, out_b, words.value)


def _out_array(out, shape):
    """A caller's output array (e.g. a PinnedBuffer's) checked for shape and
    layout, or a new one."""
    if out is None:
        return np.empty(shape, dtype=np.uint64)
    if out.shape != shape or out.dtype != np.uint64 or not out.flags.c_contiguous:
        raise ValueError(f"out must be a C-contiguous uint64 array of shape {shape}")
    return out


def respond_seeded_packed_batch(crs: ServerCrs, encoded_db: EncodedDatabase, shard_ids: Sequence[int],
                                seeds: np.ndarray, b_rows: np.ndarray, out_a: np.ndarray = None,
                                out_b: np.ndarray = None):
    """Batched respond_seeded_packed: (a (n, plen), b (n, words)) with words
    plen, or 2*plen in compat mode with more than one column.  out_a (n, plen)
    and out_b (n, 2*plen) may be given (page-locked arrays copy faster)."""
    n = len(shard_ids)
    plen = crs.params.plen
    sid = np.ascontiguousarray(shard_ids, dtype=np.uint32)
    sd = np.ascontiguousarray(seeds, dtype=np.uint8)
    br = _u64(b_rows)
    out_a = _out_array(out_a, (n, plen))
    out_b = _out_array(out_b, (n, 2 * plen))
    words = C.c_uint32(0)
    _check(crs.L.inspire_respond_seeded_packed_batch(crs.h, encoded_db.h, n, _ptr(sid), _ptr(sd), _ptr(br),
                                                     _ptr(out_a), _ptr(out_b), C.byref(words)))
    return out_a, out_b[:, :words.value]


def respond_seeded_nopacking_batch(crs: ServerCrs, encoded_db: EncodedDatabase, shard_ids: Sequence[int],
                                   seeds: np.ndarray, b_rows: np.ndarray, out: np.ndarray = None) -> np.ndarray:
    """Batched respond_seeded: (n, 2, plen) combined ciphertexts, into `out`
    when given (page-locked arrays copy faster)."""
    n = len(shard_ids)
    plen = crs.params.plen
    sid = np.ascontiguousarray(shard_ids, dtype=np.uint32)
    sd = np.ascontiguousarray(seeds, dtype=np.uint8)
    br = _u64(b_rows)
    out = _out_array(out, (n, 2, plen))
    _check(crs.L.inspire_respond_seeded_nopacking_batch(crs.h, encoded_db.h, n, _ptr(sid), _ptr(sd), _ptr(br),
                                                        _ptr(out)))
    return out


def respond_with_variant(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery,
                         variant: InspireVariant) -> ServerResponse:
    """respond_with_variant (respond.rs:129-151)."""
    if variant == InspireVariant.NoPacking:
        return respond(crs, encoded_db, query)
    if query.packing_mode == "tree":
        return respond_one_packing(crs, encoded_db, query)
    if query.inspiring_packing_keys is None:
        raise PirError("InspiRING packing keys missing (set packing_mode=tree to use tree packing)",
                       nat.ERR_KEYS_MISSING)
    return respond_inspiring(crs, encoded_db, query)


def respond_seeded_with_variant(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededClientQuery,
                                variant: InspireVariant) -> ServerResponse:
    """respond_seeded_with_variant (respond.rs:161-183)."""
    if variant == InspireVariant.NoPacking:
        return respond_seeded(crs, encoded_db, query)
    if query.packing_mode == "tree":
        return respond_seeded_packed(crs, encoded_db, query)
    if query.inspiring_packing_keys is None:
        raise PirError("InspiRING packing keys missing (set packing_mode=tree to use tree packing)",
                       nat.ERR_KEYS_MISSING)
    return respond_seeded_inspiring(crs, encoded_db, query)


def respond_seeded_batch(crs: ServerCrs, encoded_db: EncodedDatabase, shard_ids: Sequence[int], seeds: np.ndarray,
                         b_rows: np.ndarray, client_ids: Sequence[int], out: np.ndarray = None) -> np.ndarray:
    """Batched respond_seeded_inspiring with registered client keys.

    seeds (n, 2*ell, 32) uint8; b_rows (n, 2*ell, plen) uint64; returns
    (n, 2, plen) uint64 = the (a, b) of each response, in `out` when given.
    With page-locked b_rows and out (e.g. PinnedBuffer arrays) the GPU reads
    the rows and writes the responses in place, without staging copies."""
    n = len(shard_ids)
    plen = crs.params.plen
    sid = np.ascontiguousarray(shard_ids, dtype=np.uint32)
    cid = np.ascontiguousarray(client_ids, dtype=np.int32)
    sd = np.ascontiguousarray(seeds, dtype=np.uint8)
    br = _u64(b_rows)
    out = _out_array(out, (n, 2, plen))
    _check(crs.L.inspire_respond_seeded_batch(crs.h, encoded_db.h, n, _ptr(sid), _ptr(sd), _ptr(br), _ptr(cid),
                                              _ptr(out)))
    return out


def respond_batch(crs: ServerCrs, encoded_db: EncodedDatabase, shard_ids: Sequence[int], rgsw: np.ndarray,
                  client_ids: Sequence[int]) -> np.ndarray:
    """Batched respond_inspiring (full queries, respond.rs:284-386) with
    registered client keys: rgsw (n, 2*ell, 2, plen); returns (n, 2, plen)."""
    n = len(shard_ids)
    plen = crs.params.plen
    sid = np.ascontiguousarray(shard_ids, dtype=np.uint32)
    cid = np.ascontiguousarray(client_ids, dtype=np.int32)
    rg = _u64(rgsw)
    out = np.zeros((n, 2, plen), dtype=np.uint64)
    _check(crs.L.inspire_respond_batch(crs.h, encoded_db.h, n, _ptr(sid), _ptr(rg), _ptr(cid), _ptr(out)))
    return out


def respond_seeded_batch_device(crs: ServerCrs, encoded_db: EncodedDatabase, n: int, d_shard_ids: int, d_seeds: int,
                                d_b_rows: int, d_client_ids: int, d_out: int, d_status: int, stream: int,
                                max_ctas: int = 0) -> None:
    """Device-buffer batch (raw device pointers as ints); asynchronous.
    max_ctas > 0 caps the grid (each CTA then answers several queries)."""
    v = C.c_void_p
    if max_ctas:
        _check(crs.L.inspire_respond_seeded_batch_device_grid(crs.h, encoded_db.h, n, v(d_shard_ids), v(d_seeds),
                                                              v(d_b_rows), v(d_client_ids), v(d_out), v(d_status),
                                                              max_ctas, v(stream)))
        return
    _check(crs.L.inspire_respond_seeded_batch_device(crs.h, encoded_db.h, n, v(d_shard_ids), v(d_seeds), v(d_b_rows),
                                                     v(d_client_ids), v(d_out), v(d_status), v(stream)))


def ntt_forward_device(crs: ServerCrs, d_polys: int, npolys: int, stream: int) -> None:
    """Batched NttContext::forward (ntt.rs:223-246) on device u32 data."""
    _check(crs.L.inspire_ntt_forward_device(crs.h, C.c_void_p(d_polys), npolys, C.c_void_p(stream)))


def ntt_inverse_device(crs: ServerCrs, d_polys: int, npolys: int, stream: int) -> None:
    """Batched NttContext::inverse (ntt.rs:308-325) on device u32 data."""
    _check(crs.L.inspire_ntt_inverse_device(crs.h, C.c_void_p(d_polys), npolys, C.c_void_p(stream)))


def extract_inspiring_device(crs: ServerCrs, d_sk: int, d_ct: int, n: int, entry_size: int, d_entries: int,
                             stream: int) -> None:
    """decrypt + extract_inspiring (extract.rs:155-182) of n responses on the
    device (raw device pointers as ints); asynchronous."""
    v = C.c_void_p
    _check(crs.L.inspire_extract_inspiring_device(crs.h, v(d_sk), v(d_ct), n, entry_size, v(d_entries), v(stream)))


def query_seeded_device(crs: ServerCrs, d_sk: int, key: bytes, first_query: int, n: int, d_local_idx: int,
                        d_seeds: int, d_b_rows: int, d_status: int, stream: int) -> None:
    """n seeded queries (query_seeded, query.rs:43-85) of the local indices
    at d_local_idx under the secret key d_sk, generated on the device from a
    ChaCha20 stream keyed by `key` (raw device pointers as ints); outputs
    seeds [n][6][32], b_rows [n][6][2*ring_dim] (u64) and status [n] (i32);
    asynchronous."""
    if len(key) != 32:
        raise ValueError("key must be 32 bytes")
    v = C.c_void_p
    _check(crs.L.inspire_query_seeded_device(crs.h, v(d_sk), bytes(key), first_query, n, v(d_local_idx), v(d_seeds),
                                             v(d_b_rows), v(d_status), v(stream)))


def client_keygen_device(crs: ServerCrs, key: bytes, first_client: int, n: int, d_sk: int, d_y_body: int,
                         stream: int) -> None:
    """Secret keys (RlweSecretKey::generate, enc.rs:14-17) and packing key
    bodies (ClientPackingKeys::generate, inspiring2.rs:640-660) of n clients,
    generated on the device from a ChaCha20 stream keyed by `key` (raw device
    pointers as ints); d_sk [n][2*ring_dim], d_y_body [n][3][2*ring_dim]
    (u64); asynchronous."""
    if len(key) != 32:
        raise ValueError("key must be 32 bytes")
    v = C.c_void_p
    _check(crs.L.inspire_client_keygen_device(crs.h, bytes(key), first_client, n, v(d_sk), v(d_y_body), v(stream)))


def respond_seeded_packed_noalloc_device(crs: ServerCrs, encoded_db: EncodedDatabase, n: int, d_shard_ids: int,
                                         d_seeds: int, d_b_rows: int, d_out_a: int, d_out_b: int, d_status: int,
                                         stream: int) -> int:
    """Tree packing of n <= 2 seeded queries on device buffers without
    allocating (static device scratch; overlapping calls race on it, see
    include/inspire_gpu.h); asynchronous on `stream`.  Returns the b words
    per query."""
    v = C.c_void_p
    words = C.c_uint32(0)
    _check(crs.L.inspire_respond_seeded_packed_noalloc_device(crs.h, encoded_db.h, n, v(d_shard_ids), v(d_seeds),
                                                              v(d_b_rows), v(d_out_a), v(d_out_b), v(d_status),
                                                              C.byref(words), v(stream)))
    return words.value


def galois_keygen_device(crs: ServerCrs, key: bytes, d_sk: int, d_keys: int, d_status: int, stream: int) -> None:
    """The log2(d) Galois key-switching matrices of the secret key at d_sk
    (setup.rs:164-173), generated on the device from a ChaCha20 stream keyed
    by `key`; d_keys [log2 d][6][2*ring_dim] (u64), d_status [log2 d] (i32);
    asynchronous."""
    if len(key) != 32:
        raise ValueError("key must be 32 bytes")
    v = C.c_void_p
    _check(crs.L.inspire_galois_keygen_device(crs.h, bytes(key), v(d_sk), v(d_keys), v(d_status), v(stream)))


def setup_keygen_device(crs: ServerCrs, key: bytes, d_sk: int, d_ks: int, d_crs_a: int, d_status: int,
                        stream: int) -> None:
    """setup's public keys (setup.rs:151-200) of the secret key at d_sk, on the
    device: d_ks [log2 d + 4][6][2*ring_dim] (u64) = galois_keys, k_g, k_h,
    packing_k_g, packing_k_h; d_crs_a [ring_dim][2*ring_dim] (u64, 0 to skip)
    = crs_a_vectors; d_status [log2 d + 5] (i32); asynchronous."""
    if len(key) != 32:
        raise ValueError("key must be 32 bytes")
    v = C.c_void_p
    _check(crs.L.inspire_setup_keygen_device(crs.h, bytes(key), v(d_sk), v(d_ks), v(d_crs_a), v(d_status),
                                             v(stream)))


def mulmod_rate_device(crs: ServerCrs, blocks: int, iters: int, d_sink: int, stream: int) -> int:
    """Launch the modular-multiply rate probe; returns the multiplies issued."""
    _check(crs.L.inspire_mulmod_rate_device(crs.h, blocks, iters, C.c_void_p(d_sink), C.c_void_p(stream)))
    return blocks * 256 * 8 * iters


def int8_mma_rate_device(crs: ServerCrs, blocks: int, iters: int, d_a: int, d_b: int, d_out: int, stream: int) -> int:
    """INT8 tensor-core probe (mma.sync m16n8k32 s8): returns the integer
    operations issued (blocks * 8 warps * 4 chains * iters * 8192)."""
    _check(crs.L.inspire_int8_mma_rate_device(crs.h, blocks, iters, C.c_void_p(d_a), C.c_void_p(d_b),
                                              C.c_void_p(d_out), C.c_void_p(stream)))
    return blocks * 8 * 4 * iters * 8192


def external_product_device(crs: ServerCrs, d_ct: int, d_rgsw: int, d_out: int, npairs: int, stream: int) -> None:
    """Batched external_product (external_product.rs:88-150) on device u32 data."""
    _check(crs.L.inspire_external_product_device(crs.h, C.c_void_p(d_ct), C.c_void_p(d_rgsw), C.c_void_p(d_out),
                                                 npairs, C.c_void_p(stream)))


def write_crs_json(path: str, params: InspireParams, *, k_g: np.ndarray, k_h: np.ndarray, galois_keys: np.ndarray,
                   crs_a_vectors: np.ndarray, inspiring_w_seed: bytes, inspiring_v_seed: bytes,
                   inspiring_num_columns: int, packing_k_g: Optional[np.ndarray] = None,
                   packing_k_h: Optional[np.ndarray] = None, precomp: Optional[tuple] = None) -> None:
    """Write crs.json as the crate's setup binary does (serde_json of
    ServerCrs, setup.rs:52-87; bin/setup.rs:183-190).  Key-switching
    matrices have shape (gadget_len, 2, plen) rows (a, b); galois_keys
    (n, gadget_len, 2, plen); crs_a_vectors (n, plen); precomp = (a_hat,
    bold_t) from ServerCrs.inspiring_precomp or None."""
    L = nat.load()
    ell, plen = params.gadget_len, params.plen
    keep = []

    def arr(a, shape):
        if a is None:
            return None
        a = _u64(a).reshape(shape)
        keep.append(a)
        return a.ctypes.data_as(C.c_void_p)

    gk = _u64(galois_keys).reshape(-1, ell, 2, plen)
    ca = _u64(crs_a_vectors).reshape(-1, plen)
    parts = nat.ServerCrsPartsC()
    parts.k_g = arr(k_g, (ell, 2, plen))
    parts.k_h = arr(k_h, (ell, 2, plen))
    parts.galois_keys = arr(gk, gk.shape)
    parts.n_galois = gk.shape[0]
    parts.crs_a_vectors = arr(ca, ca.shape)
    parts.n_crs_a = ca.shape[0]
    parts.packing_k_g = arr(packing_k_g, (ell, 2, plen))
    parts.packing_k_h = arr(packing_k_h, (ell, 2, plen))
    if precomp is not None:
        parts.precomp_a_hat = arr(precomp[0], (plen,))
        if inspiring_num_columns > 1:
            parts.precomp_bold_t = arr(precomp[1], ((inspiring_num_columns - 1) * ell, plen))
    if len(inspiring_w_seed) != 32 or len(inspiring_v_seed) != 32:
        raise ValueError("seeds must be 32 bytes")
    parts.inspiring_w_seed[:] = list(bytes(inspiring_w_seed))
    parts.inspiring_v_seed[:] = list(bytes(inspiring_v_seed))
    parts.inspiring_num_columns = int(inspiring_num_columns)
    pc = params.to_c()
    _check(L.inspire_crs_write_json(C.byref(pc), C.byref(parts), str(path).encode()))


def now_ns() -> int:
    """The serving loop's clock (CLOCK_MONOTONIC, ns)."""
    return int(nat.load().inspire_now_ns())


class Server:
    """Serving loop over one ServerCrs: continuous batching of seeded
    InspiRING queries (the GPU replacement of the crate's per-request
    respond call in src/bin/server.rs:179-236).

    submit() copies each query's rows into a pinned slot and returns tickets;
    a native dispatcher launches pending queries in batches of up to
    max_batch on max_inflight streams as they free up; poll() collects a
    response.  Client keys are those registered with
    ServerCrs.register_client; queries may name any database of the CRS."""

    def __init__(self, crs: ServerCrs, max_batch: int = 128, max_inflight: int = 4, capacity: int = 4096,
                 device_budget: int = 0, batch_wait_us: int = 100, stage_wait_iters: Optional[int] = None):
        self.crs = crs
        self.L = crs.L
        cfg = nat.ServerConfigC()
        self.L.inspire_server_config_default(C.byref(cfg))
        cfg.max_batch, cfg.max_inflight, cfg.capacity, cfg.device_budget = max_batch, max_inflight, capacity, \
            device_budget
        cfg.batch_wait_us = batch_wait_us
        if stage_wait_iters is not None:
            cfg.stage_wait_iters = stage_wait_iters
        h = C.c_void_p()
        _check(self.L.inspire_server_create(crs.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self.plen = crs.params.plen
        _LIVE_SERVERS.add(self)

    def submit(self, encoded_db, shard_ids, seeds: np.ndarray, b_rows: np.ndarray, client_ids,
               arrival_ns: Optional[np.ndarray] = None, borrow: bool = False):
        """Submit n queries (seeds (n, 2*ell, 32), b_rows (n, 2*ell, plen));
        encoded_db is one EncodedDatabase for all of them or a sequence of n.
        borrow=True reads the rows in place (they must lie in PinnedBuffer
        memory and stay unchanged until collected).  Returns (tickets,
        status): tickets of the accepted prefix, status 0, ERR_BUSY (capacity
        reached) or the error of the first invalid query (raised as PirError
        when nothing was accepted)."""
        sid = np.ascontiguousarray(shard_ids, dtype=np.uint32)
        n = sid.size
        if isinstance(encoded_db, EncodedDatabase):
            dbs = np.full(n, encoded_db.h.value, dtype=np.uint64)
        elif isinstance(encoded_db, np.ndarray):  # handle values (Server.handle_of)
            dbs = np.ascontiguousarray(encoded_db, dtype=np.uint64)
        else:
            dbs = np.array([d.h.value for d in encoded_db], dtype=np.uint64)
        if dbs.size != n:
            raise ValueError("one database per query")
        cid = np.ascontiguousarray(client_ids, dtype=np.int32)
        if borrow:
            sd, br = seeds, b_rows
            if not (sd.flags.c_contiguous and br.flags.c_contiguous and sd.dtype == np.uint8 and
                    br.dtype == np.uint64):
                raise ValueError("borrowed rows must be C-contiguous uint8 seeds / uint64 b_rows")
        else:
            sd = np.ascontiguousarray(seeds, dtype=np.uint8)
            br = _u64(b_rows)
        arr = None if arrival_ns is None else np.ascontiguousarray(arrival_ns, dtype=np.int64)
        tickets = np.zeros(n, dtype=np.uint64)
        acc = C.c_uint32(0)
        rc = self.L.inspire_server_submit(self.h, n, _ptr(dbs), _ptr(sid), _ptr(sd), _ptr(br), _ptr(cid), _ptr(arr),
                                          nat.SUBMIT_BORROW if borrow else 0, _ptr(tickets), C.byref(acc))
        if rc not in (nat.OK, nat.ERR_BUSY) and acc.value == 0:
            raise PirError(nat.last_error(), rc)
        return tickets[:acc.value], rc

    @staticmethod
    def handle_of(encoded_db: EncodedDatabase) -> int:
        """The native handle value submit() accepts in a uint64 array."""
        return int(encoded_db.h.value)

    def poll(self, ticket: int, out: Optional[np.ndarray] = None, timeout_us: int = -1):
        """Collect one ticket.  Returns done_ns when ready (out, if given,
        receives (2, plen) uint64), None if still pending after timeout_us."""
        done = C.c_int64(0)
        rc = self.L.inspire_server_poll(self.h, int(ticket), _ptr(out), C.byref(done), int(timeout_us))
        if rc == nat.PENDING:
            return None
        _check(rc)
        return int(done.value)

    def poll_batch(self, tickets: np.ndarray, out: Optional[np.ndarray] = None, timeout_us: int = -1):
        """Collect tickets in order (out, if given: (n, 2, plen) uint64).
        Returns done_ns of the collected prefix (shorter than tickets if one
        is still pending after timeout_us)."""
        tk = np.ascontiguousarray(tickets, dtype=np.uint64)
        done = np.zeros(tk.size, dtype=np.int64)
        got = C.c_uint32(0)
        rc = self.L.inspire_server_poll_batch(self.h, tk.size, _ptr(tk), _ptr(out), _ptr(done), int(timeout_us),
                                              C.byref(got))
        if rc not in (nat.OK, nat.PENDING):
            raise PirError(nat.last_error(), rc)
        return done[:got.value]

    def drive(self, db_handles, shard_ids, client_ids, pool_seeds: np.ndarray, pool_b_rows: np.ndarray,
              arrival_ns: np.ndarray, borrow: bool = False, max_burst: int = 256, n_keep: int = 0):
        """Open-loop load driven natively (inspire_server_drive): query k is
        submitted at arrival_ns[k] (now_ns clock, non-decreasing) with the
        rows of pool entry k mod len(pool_seeds), by a native thread spinning
        on the clock; a second native thread collects.  db_handles
        (handle_of values), shard_ids and client_ids are per query.  Returns
        (submit_ns, done_ns, responses of the first n_keep queries or None).
        A rejected query, or one that fails on the device, stops the
        submissions and raises PirError with the first error, after every
        query accepted until then has been collected."""
        arr = np.ascontiguousarray(arrival_ns, dtype=np.int64)
        n = arr.size
        dbs = np.ascontiguousarray(db_handles, dtype=np.uint64)
        sid = np.ascontiguousarray(shard_ids, dtype=np.uint32)
        cid = np.ascontiguousarray(client_ids, dtype=np.int32)
        if dbs.size != n or sid.size != n or cid.size != n:
            raise ValueError("one database, shard and client per query")
        if borrow:
            sd, br = pool_seeds, pool_b_rows
            if not (sd.flags.c_contiguous and br.flags.c_contiguous and sd.dtype == np.uint8 and
                    br.dtype == np.uint64):
                raise ValueError("borrowed rows must be C-contiguous uint8 seeds / uint64 b_rows")
        else:
            sd = np.ascontiguousarray(pool_seeds, dtype=np.uint8)
            br = _u64(pool_b_rows)
        submit = np.zeros(n, dtype=np.int64)
        done = np.zeros(n, dtype=np.int64)
        keep = np.zeros((n_keep, 2, self.plen), dtype=np.uint64) if n_keep else None
        _check(self.L.inspire_server_drive(self.h, n, _ptr(dbs), _ptr(sid), _ptr(cid), _ptr(sd), _ptr(br),
                                           sd.shape[0], _ptr(arr), nat.SUBMIT_BORROW if borrow else 0, max_burst,
                                           _ptr(submit), _ptr(done), n_keep, _ptr(keep)))
        return submit, done, keep

    def stats(self) -> dict:
        st = nat.ServerStatsC()
        _check(self.L.inspire_server_get_stats(self.h, C.byref(st)))
        return {k: int(getattr(st, k)) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.L.inspire_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked, device-mapped host memory (inspire_pinned_alloc) viewed
    as a numpy array; the serving loop can read borrowed query rows from it
    in place."""

    def __init__(self, shape, dtype):
        self.L = nat.load()
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        p = C.c_void_p()
        _check(self.L.inspire_pinned_alloc(nbytes, C.byref(p)))
        self.p = p
        raw = (C.c_uint8 * nbytes).from_address(p.value)
        self.array = np.frombuffer(raw, dtype=np.uint8).view(dt).reshape(shape)
        _LIVE_PINNED.add(self)

    def close(self):
        if getattr(self, "p", None):
            self.array = None
            self.L.inspire_pinned_free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
