"""ctypes binding of libinspire_gpu.so (the C ABI in include/inspire_gpu.h).

The library is built in-tree by inspire-rs_gb300/build_lib.py.  There is no
CPU implementation behind this module: if the library is missing or cannot be
loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libinspire_gpu.so")
HEADER = os.path.join(os.path.dirname(PKG_ROOT), "include", "inspire_gpu.h")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_SHARD_NOT_FOUND = 2
ERR_KEYS_MISSING = 3
ERR_KEYS_INVALID = 4
ERR_UNSUPPORTED = 5
ERR_CUDA = 6
ERR_OUT_OF_MEMORY = 7
ERR_NO_CRS = 8
ERR_DEVICE_STATUS = 9
PENDING = 10
ERR_BUSY = 11
SUBMIT_BORROW = 1

MODE_COMPAT = 0
MODE_CRT_FIXED = 1


class InspireParamsC(C.Structure):
    _fields_ = [
        ("ring_dim", C.c_uint32),
        ("crt_count", C.c_uint32),
        ("crt_moduli", C.c_uint64 * 2),
        ("p", C.c_uint64),
        ("sigma", C.c_double),
        ("gadget_base", C.c_uint64),
        ("gadget_len", C.c_uint32),
    ]


class ServerCrsPartsC(C.Structure):
    _fields_ = [
        ("k_g", C.c_void_p),
        ("k_h", C.c_void_p),
        ("galois_keys", C.c_void_p),
        ("n_galois", C.c_uint32),
        ("crs_a_vectors", C.c_void_p),
        ("n_crs_a", C.c_uint32),
        ("packing_k_g", C.c_void_p),
        ("packing_k_h", C.c_void_p),
        ("precomp_a_hat", C.c_void_p),
        ("precomp_bold_t", C.c_void_p),
        ("inspiring_w_seed", C.c_uint8 * 32),
        ("inspiring_v_seed", C.c_uint8 * 32),
        ("inspiring_num_columns", C.c_uint32),
    ]


class HttpConfigC(C.Structure):
    _fields_ = [
        ("host", C.c_char_p),
        ("port", C.c_uint16),
        ("max_clients", C.c_uint32),
        ("max_body", C.c_uint64),
        ("version", C.c_char_p),
        ("entry_count", C.c_uint64),
        ("shard_count", C.c_uint64),
    ]


class SeededQueryC(C.Structure):
    _fields_ = [
        ("shard_id", C.c_uint32),
        ("seeds", C.c_void_p),
        ("b_rows", C.c_void_p),
        ("has_packing_keys", C.c_int32),
        ("y_body", C.c_void_p),
        ("y_all", C.c_void_p),
    ]


class QueryC(C.Structure):
    _fields_ = [
        ("shard_id", C.c_uint32),
        ("rgsw", C.c_void_p),
        ("has_packing_keys", C.c_int32),
        ("y_body", C.c_void_p),
        ("y_all", C.c_void_p),
    ]


class ServerConfigC(C.Structure):
    _fields_ = [
        ("max_batch", C.c_uint32),
        ("max_inflight", C.c_uint32),
        ("capacity", C.c_uint32),
        ("device_budget", C.c_uint64),
        ("batch_wait_us", C.c_uint32),
        ("stage_wait_iters", C.c_uint32),
    ]


class ServerStatsC(C.Structure):
    _fields_ = [
        ("submitted", C.c_uint64),
        ("completed", C.c_uint64),
        ("batches", C.c_uint64),
        ("pending", C.c_uint32),
        ("inflight_batches", C.c_uint32),
        ("streams", C.c_uint32),
    ]


_lib = None


def load(path: str = LIB_PATH):
    """Load the native library (raises OSError if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"libinspire_gpu.so not built: {path} (run inspire-rs_gb300/build_lib.py)")
    L = C.CDLL(path)
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32
    sig = {
        "inspire_last_error": (C.c_char_p, []),
        "inspire_version": (C.c_char_p, []),
        "inspire_params_default": (None, [C.POINTER(InspireParamsC)]),
        "inspire_ctx_create": (C.c_int, [C.POINTER(InspireParamsC), C.c_int, C.c_int, C.POINTER(vp)]),
        "inspire_ctx_destroy": (None, [vp]),
        "inspire_crs_load": (C.c_int, [vp, vp, u32]),
        "inspire_db_create": (C.c_int, [vp, vp, u64, u32, C.POINTER(vp)]),
        "inspire_db_destroy": (None, [vp]),
        "inspire_db_load_shards": (C.c_int, [vp, C.c_char_p, C.POINTER(vp)]),
        "inspire_db_load_json": (C.c_int, [vp, C.c_char_p, C.c_size_t, C.POINTER(vp)]),
        "inspire_crs_load_json": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
        "inspire_crs_info": (C.c_int, [vp, vp, C.POINTER(u32), C.POINTER(i32)]),
        "inspire_db_save_shards": (C.c_int, [vp, C.POINTER(InspireParamsC), C.c_char_p]),
        "inspire_db_num_shards": (u32, [vp]),
        "inspire_db_device_bytes": (u64, [vp]),
        "inspire_client_register": (C.c_int, [vp, vp, vp, C.POINTER(i32)]),
        "inspire_client_release": (C.c_int, [vp, i32]),
        "inspire_respond_seeded_inspiring": (C.c_int, [vp, vp, C.POINTER(SeededQueryC), vp]),
        "inspire_respond_inspiring": (C.c_int, [vp, vp, C.POINTER(QueryC), vp]),
        "inspire_respond": (C.c_int, [vp, vp, C.POINTER(QueryC), vp, vp]),
        "inspire_respond_seeded": (C.c_int, [vp, vp, C.POINTER(SeededQueryC), vp, vp]),
        "inspire_respond_seeded_nopacking_batch": (C.c_int, [vp, vp, u32, vp, vp, vp, vp]),
        "inspire_respond_seeded_batch": (C.c_int, [vp, vp, u32, vp, vp, vp, vp, vp]),
        "inspire_respond_batch": (C.c_int, [vp, vp, u32, vp, vp, vp, vp]),
        "inspire_respond_seeded_batch_device": (C.c_int, [vp, vp, u32, vp, vp, vp, vp, vp, vp, vp]),
        "inspire_respond_seeded_batch_device_grid": (C.c_int, [vp, vp, u32, vp, vp, vp, vp, vp, vp, u32, vp]),
        "inspire_server_config_default": (None, [C.POINTER(ServerConfigC)]),
        "inspire_server_create": (C.c_int, [vp, C.POINTER(ServerConfigC), C.POINTER(vp)]),
        "inspire_server_destroy": (None, [vp]),
        "inspire_server_submit": (C.c_int, [vp, u32, vp, vp, vp, vp, vp, vp, u32, vp, C.POINTER(u32)]),
        "inspire_pinned_alloc": (C.c_int, [C.c_size_t, C.POINTER(vp)]),
        "inspire_pinned_free": (None, [vp]),
        "inspire_server_poll": (C.c_int, [vp, u64, vp, C.POINTER(C.c_int64), i32]),
        "inspire_server_poll_batch": (C.c_int, [vp, u32, vp, vp, vp, i32, C.POINTER(u32)]),
        "inspire_server_drive": (C.c_int, [vp, u32, vp, vp, vp, vp, vp, u32, vp, u32, u32, vp, vp, u32, vp]),
        "inspire_server_get_stats": (C.c_int, [vp, C.POINTER(ServerStatsC)]),
        "inspire_now_ns": (C.c_int64, []),
        "inspire_mulmod_rate_device": (C.c_int, [vp, u32, u32, vp, vp]),
        "inspire_int8_mma_rate_device": (C.c_int, [vp, u32, u32, vp, vp, vp, vp]),
        "inspire_extract_inspiring_device": (C.c_int, [vp, vp, vp, u32, u32, vp, vp]),
        "inspire_query_seeded_device": (C.c_int, [vp, vp, C.c_char_p, u64, u32, vp, vp, vp, vp, vp]),
        "inspire_crs_load_galois_keys": (C.c_int, [vp, vp, u32]),
        "inspire_respond_one_packing": (C.c_int, [vp, vp, C.POINTER(QueryC), vp, vp, C.POINTER(u32)]),
        "inspire_respond_seeded_packed": (C.c_int, [vp, vp, C.POINTER(SeededQueryC), vp, vp, C.POINTER(u32)]),
        "inspire_respond_seeded_packed_batch": (C.c_int, [vp, vp, u32, vp, vp, vp, vp, vp, C.POINTER(u32)]),
        "inspire_galois_keygen_device": (C.c_int, [vp, C.c_char_p, vp, vp, vp, vp]),
        "inspire_setup_keygen_device": (C.c_int, [vp, C.c_char_p, vp, vp, vp, vp, vp]),
        "inspire_respond_seeded_packed_noalloc_device": (C.c_int, [vp, vp, u32, vp, vp, vp, vp, vp, vp,
                                                                   C.POINTER(u32), vp]),
        "inspire_client_keygen_device": (C.c_int, [vp, C.c_char_p, u64, u32, vp, vp, vp]),
        "inspire_seeded_query_from_json": (C.c_int, [C.POINTER(InspireParamsC), C.c_char_p, C.c_size_t, vp, vp, vp,
                                                     vp, vp, vp]),
        "inspire_query_response_to_json": (C.c_int, [C.POINTER(InspireParamsC), vp, u32, vp, u64, vp, C.c_size_t,
                                                     C.POINTER(C.c_size_t)]),
        "inspire_query_from_json": (C.c_int, [C.POINTER(InspireParamsC), C.c_char_p, C.c_size_t, vp, vp, vp, vp,
                                              vp]),
        "inspire_packed_response_to_json": (C.c_int, [C.POINTER(InspireParamsC), vp, vp, u32, u64, vp,
                                                      C.c_size_t, C.POINTER(C.c_size_t)]),
        "inspire_crs_write_json": (C.c_int, [C.POINTER(InspireParamsC), C.POINTER(ServerCrsPartsC), C.c_char_p]),
        "inspire_crs_a_vectors_count": (u64, [vp]),
        "inspire_inspiring_precomp": (C.c_int, [vp, vp, vp, vp]),
        "inspire_ctx_set_device_budget": (C.c_int, [vp, u64]),
        "inspire_ctx_set_pair_threshold": (C.c_int, [vp, u32]),
        "inspire_ctx_pair_threshold": (u32, [vp]),
        "inspire_http_config_default": (None, [C.POINTER(HttpConfigC)]),
        "inspire_http_start": (C.c_int, [vp, vp, vp, C.POINTER(HttpConfigC), C.c_char_p, C.c_size_t,
                                         C.POINTER(vp)]),
        "inspire_http_port": (C.c_uint16, [vp]),
        "inspire_http_stop": (None, [vp]),
        "inspire_ctx_device_memory": (C.c_int, [vp, C.POINTER(u64), C.POINTER(u64)]),
        "inspire_server_response_to_bincode": (C.c_int, [C.POINTER(InspireParamsC), vp, u32, vp, vp, C.c_size_t,
                                                         C.POINTER(C.c_size_t)]),
        "inspire_ntt_forward_device": (C.c_int, [vp, vp, u32, vp]),
        "inspire_ntt_inverse_device": (C.c_int, [vp, vp, u32, vp]),
        "inspire_external_product_device": (C.c_int, [vp, vp, vp, vp, u32, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return load().inspire_last_error().decode()


def declared_symbols(header: str = HEADER) -> list[str]:
    """Names of the functions declared in include/inspire_gpu.h."""
    import re

    text = open(header).read()
    return sorted(set(re.findall(r"\b(inspire_[a-z0-9_]+)\s*\(", text)))
