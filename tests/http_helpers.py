"""Shared pieces of the HTTP tests: the crate's JSON bodies built from its
serde derives (ClientQuery, SeededClientQuery, ClientPackingKeys, Poly) and
a small HTTP client."""
import http.client
import json

import numpy as np

N = 2048
Q = (268369921, 249561089)
QC = Q[0] * Q[1]
QINV = pow(Q[0], Q[1] - 2, Q[1])


def poly_obj(coeffs):
    return {"coeffs": [int(x) for x in coeffs], "moduli": list(Q), "q": QC, "dim": N, "crt_q0_inv_mod_q1": QINV,
            "is_ntt": False}


def keys_obj(y_body):
    return {"y_body": [poly_obj(p) for p in y_body], "full_key": False, "num_to_pack": 16}


def seeded_query_body(shard_id, seeds, b_rows, y_body=None, mode="inspiring"):
    q = {"shard_id": int(shard_id),
         "rgsw_ciphertext": {"rows": [{"seed": [int(v) for v in seeds[i]], "b": poly_obj(b_rows[i])}
                                      for i in range(6)],
                             "gadget": {"base": 1 << 20, "len": 3, "q": QC}},
         "packing_mode": mode}
    if y_body is not None:
        q["inspiring_packing_keys"] = keys_obj(y_body)
    return json.dumps(q, separators=(",", ":")).encode()


def full_query_body(shard_id, rgsw, y_body=None, mode="inspiring"):
    rows = np.asarray(rgsw).reshape(6, 2, 2 * N)
    q = {"shard_id": int(shard_id),
         "rgsw_ciphertext": {"rows": [{"a": poly_obj(rows[i, 0]), "b": poly_obj(rows[i, 1])} for i in range(6)],
                             "gadget": {"base": 1 << 20, "len": 3, "q": QC}},
         "packing_mode": mode}
    if y_body is not None:
        q["inspiring_packing_keys"] = keys_obj(y_body)
    return json.dumps(q, separators=(",", ":")).encode()


def request(url_or_conn, method, path, body=None, ctype="application/json"):
    """(status, content-type, body bytes) of one request."""
    if isinstance(url_or_conn, http.client.HTTPConnection):
        conn, own = url_or_conn, False
    else:
        host, port = url_or_conn.split("//")[1].split(":")
        conn, own = http.client.HTTPConnection(host, int(port), timeout=120), True
    headers = {} if ctype is None else {"Content-Type": ctype}
    conn.request(method, path, body=body, headers=headers)
    r = conn.getresponse()
    data = r.read()
    out = (r.status, r.getheader("content-type"), data)
    if own:
        conn.close()
    return out


def ciphertext_of(reply: bytes) -> np.ndarray:
    """(a, b) of a QueryResponse JSON reply as a (2, plen) array."""
    obj = json.loads(reply)
    ct = obj["response"]["ciphertext"]
    return np.array([ct["a"]["coeffs"], ct["b"]["coeffs"]], dtype=np.uint64)
