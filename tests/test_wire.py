"""Native wire codecs (host code, no GPU): SeededClientQuery JSON in, the
server's JSON reply and ServerResponse's bincode out.  The expected bytes are
built here from the crate's serde derives (field names and order of Poly,
SeededRlweCiphertext, SeededRgswCiphertext, GadgetVector, ClientPackingKeys,
SeededClientQuery, RlweCiphertext, ServerResponse, QueryResponse) with
serde_json's compact formatting and bincode 1.3's fixed-width little-endian
encoding."""
import json
import struct

import numpy as np
import pytest

N = 2048
Q = (268369921, 249561089)
QC = Q[0] * Q[1]
QINV = pow(Q[0], Q[1] - 2, Q[1])  # Poly::crt_q0_inv_mod_q1


@pytest.fixture(scope="module")
def wire():
    import build_lib

    build_lib.build()
    import inspire
    from inspire import wire as w

    return inspire, w


def poly_obj(coeffs):
    return {"coeffs": [int(x) for x in coeffs], "moduli": list(Q), "q": QC, "dim": N, "crt_q0_inv_mod_q1": QINV,
            "is_ntt": False}


def query_obj(shard_id, seeds, b_rows, y_body=None, mode=None, keys_null=False):
    q = {"shard_id": shard_id,
         "rgsw_ciphertext": {"rows": [{"seed": [int(b) for b in seeds[i]], "b": poly_obj(b_rows[i])}
                                      for i in range(6)],
                             "gadget": {"base": 1 << 20, "len": 3, "q": QC}}}
    if mode is not None:
        q["packing_mode"] = mode
    if y_body is not None:
        q["inspiring_packing_keys"] = {"y_body": [poly_obj(p) for p in y_body], "full_key": False, "num_to_pack": 16}
    elif keys_null:
        q["inspiring_packing_keys"] = None
    return q


def compact(obj):
    return json.dumps(obj, separators=(",", ":")).encode()


def rand_polys(rng, n):
    a = np.zeros((n, 2 * N), np.uint64)
    a[:, :N] = rng.integers(0, Q[0], size=(n, N))
    a[:, N:] = rng.integers(0, Q[1], size=(n, N))
    return a


def test_seeded_query_json_round_trip(wire):
    inspire, w = wire
    rng = np.random.default_rng(1)
    params = inspire.InspireParams(p=1 << 16)
    seeds = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
    b_rows, y_body = rand_polys(rng, 6), rand_polys(rng, 3)
    q = w.seeded_query_from_json(params, compact(query_obj(17, seeds, b_rows, y_body, mode="inspiring")))
    assert q.shard_id == 17 and q.packing_mode == "inspiring"
    assert np.array_equal(q.seeds, seeds) and np.array_equal(q.b_rows, b_rows)
    assert np.array_equal(q.inspiring_packing_keys.y_body, y_body)
    # pretty-printed, packing_mode defaulted, keys omitted / null, tree mode
    q2 = w.seeded_query_from_json(params, json.dumps(query_obj(3, seeds, b_rows), indent=2))
    assert q2.packing_mode == "inspiring" and q2.inspiring_packing_keys is None
    q3 = w.seeded_query_from_json(params, compact(query_obj(3, seeds, b_rows, mode="tree", keys_null=True)))
    assert q3.packing_mode == "tree" and q3.inspiring_packing_keys is None
    assert np.array_equal(q3.b_rows, b_rows)


def test_seeded_query_json_rejects(wire):
    inspire, w = wire
    rng = np.random.default_rng(2)
    params = inspire.InspireParams(p=1 << 16)
    seeds = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
    b_rows = rand_polys(rng, 6)
    good = query_obj(1, seeds, b_rows)
    cases = []
    o = json.loads(compact(good))
    o["rgsw_ciphertext"]["rows"] = o["rgsw_ciphertext"]["rows"][:5]
    cases.append((o, "2\\*gadget_len"))
    o = json.loads(compact(good))
    o["rgsw_ciphertext"]["rows"][2]["b"]["moduli"] = [12289, 40961]
    cases.append((o, "moduli"))
    o = json.loads(compact(good))
    o["rgsw_ciphertext"]["rows"][0]["b"]["is_ntt"] = True
    cases.append((o, "coefficient form"))
    o = json.loads(compact(good))
    o["rgsw_ciphertext"]["rows"][0]["seed"] = o["rgsw_ciphertext"]["rows"][0]["seed"][:31]
    cases.append((o, "32 bytes"))
    o = json.loads(compact(good))
    o["rgsw_ciphertext"]["rows"][1]["b"]["coeffs"][0] = Q[0]
    cases.append((o, "not reduced"))
    o = json.loads(compact(good))
    o["packing_mode"] = "fancy"
    cases.append((o, "packing_mode"))
    o = json.loads(compact(good))
    o["rgsw_ciphertext"]["gadget"]["base"] = 1 << 16
    cases.append((o, "gadget"))
    for obj, msg in cases:
        with pytest.raises(inspire.PirError, match=msg):
            w.seeded_query_from_json(params, compact(obj))
    with pytest.raises(inspire.PirError, match="trailing"):
        w.seeded_query_from_json(params, compact(good) + b" x")
    with pytest.raises(inspire.PirError, match="expected"):
        w.seeded_query_from_json(params, compact(good)[:-10])


def test_seeded_query_json_number_forms(wire):
    """Integer arrays in every form the parser meets: 1..9-digit values,
    whitespace around values and commas, values at the end of an array, and
    over-long, overflowing and non-integer numbers (the compact form is
    parsed eight bytes at a time, everything else by the checked path)."""
    inspire, w = wire
    rng = np.random.default_rng(3)
    params = inspire.InspireParams(p=1 << 16)
    seeds = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
    b_rows = rand_polys(rng, 6)
    # row 0's coefficients with 1..9 digits each, row 1 with random spacing
    for i in range(2 * N):
        nd = 1 + i % 9
        b_rows[0, i] = int(rng.integers(10 ** (nd - 1) if nd > 1 else 0, min(10 ** nd, Q[i // N])))
    good = compact(query_obj(1, seeds, b_rows))
    spaced = ",".join(rng.choice(["", " ", "\n", "  \t"]) + str(int(v)) + rng.choice(["", " ", "\r\n"])
                      for v in b_rows[1])
    body = good.replace(b'"coeffs":[' + ",".join(str(int(v)) for v in b_rows[1]).encode() + b"]",
                        b'"coeffs":[' + spaced.encode() + b"]")
    assert body != good
    for text in (good, body):
        q = w.seeded_query_from_json(params, text)
        assert np.array_equal(q.b_rows, b_rows)
    first = str(int(b_rows[2, 0])).encode()
    key = b'"coeffs":[' + first + b","
    assert good.count(key) == 1
    bad = [(b"1234567890123456", "not reduced"), (b"99999999999999999", "not reduced"),
           (b"18446744073709551615", "not reduced"), (b"18446744073709551616", "overflow"),
           (b"123456789012345678901", "overflow"), (b"12.5", "integer"), (b"1e3", "integer"),
           (b"-4", "unsigned"), (b"12a", "expected"),
           # serde_json rejects leading zeros: through the compact run, the
           # one-number fast path and the checked path alike
           (b"007", "leading zero"), (b"00", "leading zero"), (b"0" + first, "leading zero")]
    # every length from 10 to 16 digits is above both moduli: rejected, not
    # misparsed into a value below q
    bad += [(b"9" * n, "not reduced") for n in range(10, 17)]
    bad += [(b"1" + b"0" * (n - 1), "not reduced") for n in range(10, 17)]
    for num, msg in bad:
        with pytest.raises(inspire.PirError, match=msg):
            w.seeded_query_from_json(params, good.replace(key, b'"coeffs":[' + num + b","))
        # the same number as the last element of the array, and after a space
        last = str(int(b_rows[2, 2 * N - 1])).encode()
        lkey = b"," + last + b'],"moduli"'
        if good.count(lkey) == 1:
            with pytest.raises(inspire.PirError, match=msg):
                w.seeded_query_from_json(params, good.replace(lkey, b"," + num + b'],"moduli"'))
        with pytest.raises(inspire.PirError, match=msg):
            w.seeded_query_from_json(params, good.replace(key, b'"coeffs":[ ' + num + b","))


def test_json_number_paths_exhaustive(tmp_path):
    """The codec's three unsigned-integer paths (compact run, one-number fast
    path, checked path) give the exact value for every length from 1 to 16
    digits at every distance from the end of the buffer, and reject what
    serde_json rejects (leading zeros, signs, fractions, overflow): a C++
    driver built against json_codec.h with g++."""
    import os
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "inspire-rs_gb300", "csrc")
    exe = str(tmp_path / "json_numbers")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", csrc, os.path.join(here, "native", "json_numbers.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout


def test_response_json_and_bincode(wire):
    inspire, w = wire
    rng = np.random.default_rng(3)
    params = inspire.InspireParams(p=1 << 16)
    ct = rand_polys(rng, 2)
    cols = rand_polys(rng, 4)
    for columns in ([], [inspire.RlweCiphertext(cols[0], cols[1]), inspire.RlweCiphertext(cols[2], cols[3])]):
        resp = inspire.ServerResponse(inspire.RlweCiphertext(ct[0], ct[1]), columns)
        want = compact({"response": {"ciphertext": {"a": poly_obj(ct[0]), "b": poly_obj(ct[1])},
                                     "column_ciphertexts": [{"a": poly_obj(c.a), "b": poly_obj(c.b)} for c in columns]},
                        "processing_time_ms": 12})
        assert w.query_response_to_json(params, resp, 12) == want

        def poly_bin(c):
            return (struct.pack("<Q", 2 * N) + np.asarray(c, "<u8").tobytes() + struct.pack("<QQQ", 2, *Q) +
                    struct.pack("<QQQ", QC, N, QINV) + b"\x00")

        want_bin = poly_bin(ct[0]) + poly_bin(ct[1]) + struct.pack("<Q", len(columns)) + b"".join(
            poly_bin(c.a) + poly_bin(c.b) for c in columns)
        assert w.server_response_to_bincode(params, resp) == want_bin


def full_query_obj(shard_id, rgsw, y_body=None, mode=None, keys_empty=False):
    q = {"shard_id": shard_id,
         "rgsw_ciphertext": {"rows": [{"a": poly_obj(rgsw[i, 0]), "b": poly_obj(rgsw[i, 1])} for i in range(6)],
                             "gadget": {"base": 1 << 20, "len": 3, "q": QC}}}
    if mode is not None:
        q["packing_mode"] = mode
    if y_body is not None:
        q["inspiring_packing_keys"] = {"y_body": [poly_obj(p) for p in y_body], "full_key": False, "num_to_pack": 16}
    elif keys_empty:
        q["inspiring_packing_keys"] = {"y_body": [], "full_key": False, "num_to_pack": 16}
    return q


def test_client_query_json(wire):
    """ClientQuery (query.rs:119-132) JSON, the /query request: full RGSW rows
    (a, b), packing mode, optional keys; an empty y_body is kept as 'keys
    present, invalid' so that respond reports it as the crate does."""
    inspire, w = wire
    rng = np.random.default_rng(5)
    params = inspire.InspireParams(p=1 << 16)
    rgsw = rand_polys(rng, 12).reshape(6, 2, 2 * N)
    y_body = rand_polys(rng, 3)
    q = w.query_from_json(params, compact(full_query_obj(9, rgsw, y_body, mode="tree")))
    assert q.shard_id == 9 and q.packing_mode == "tree"
    assert np.array_equal(q.rgsw, rgsw)
    assert np.array_equal(q.inspiring_packing_keys.y_body, y_body)
    q = w.query_from_json(params, json.dumps(full_query_obj(3, rgsw), indent=1))
    assert q.packing_mode == "inspiring" and q.inspiring_packing_keys is None
    q = w.query_from_json(params, compact(full_query_obj(3, rgsw, keys_empty=True)))
    assert q.inspiring_packing_keys is not None and q.inspiring_packing_keys.y_body is None
    # the seeded parser keeps the same distinction
    seeds = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
    body = query_obj(1, seeds, rgsw[:, 1])
    body["inspiring_packing_keys"] = {"y_body": [], "full_key": False, "num_to_pack": 16}
    sq = w.seeded_query_from_json(params, compact(body))
    assert sq.inspiring_packing_keys is not None and sq.inspiring_packing_keys.y_body is None
    bad = full_query_obj(3, rgsw)
    del bad["rgsw_ciphertext"]["rows"][2]["a"]
    with pytest.raises(inspire.PirError, match="needs a and b"):
        w.query_from_json(params, compact(bad))
    bad = full_query_obj(3, rgsw)
    bad["rgsw_ciphertext"]["rows"] = bad["rgsw_ciphertext"]["rows"][:5]
    with pytest.raises(inspire.PirError, match="2\\*gadget_len"):
        w.query_from_json(params, compact(bad))


def test_packed_response_json(wire):
    """The /query reply for tree packing, with a ring_dim b and with the
    crate's compat-mode b of dimension 2 ring_dim."""
    inspire, w = wire
    rng = np.random.default_rng(6)
    params = inspire.InspireParams(p=1 << 16)
    a = rand_polys(rng, 1)[0]
    for b in (rand_polys(rng, 1)[0], np.concatenate([rand_polys(rng, 1)[0], rand_polys(rng, 1)[0]])):
        dim = b.size // 2
        pb = {"coeffs": [int(x) for x in b], "moduli": list(Q), "q": QC, "dim": dim, "crt_q0_inv_mod_q1": QINV,
              "is_ntt": False}
        want = compact({"response": {"ciphertext": {"a": poly_obj(a), "b": pb}, "column_ciphertexts": []},
                        "processing_time_ms": 7})
        assert w.packed_response_to_json(params, a, b, 7) == want


def test_crs_json_writer(wire, tmp_path):
    """crs.json as the crate's setup writes it (serde_json of ServerCrs,
    setup.rs:52-87, field order of the derive, skipped fields left out):
    built here from the derives and compared byte for byte."""
    inspire, w = wire
    rng = np.random.default_rng(7)
    params = inspire.InspireParams(p=1 << 16)
    ksm = lambda: rand_polys(rng, 6).reshape(3, 2, 2 * N)  # noqa: E731
    k_g, k_h, pk_g = ksm(), ksm(), ksm()
    galois = np.stack([ksm() for _ in range(2)])
    crs_a = rand_polys(rng, 3)
    a_hat = rand_polys(rng, 1)[0]
    bold_t = rng.integers(0, 1 << 20, size=(15 * 3, 2 * N), dtype=np.uint64)
    wseed, vseed = bytes(range(32)), bytes(range(100, 132))
    path = tmp_path / "crs.json"
    inspire.write_crs_json(str(path), params, k_g=k_g, k_h=k_h, galois_keys=galois, crs_a_vectors=crs_a,
                           inspiring_w_seed=wseed, inspiring_v_seed=vseed, inspiring_num_columns=16,
                           packing_k_g=pk_g, packing_k_h=None, precomp=(a_hat, bold_t))
    gadget = {"base": 1 << 20, "len": 3, "q": QC}

    def ksm_obj(m):
        return {"rows": [{"a": poly_obj(m[k, 0]), "b": poly_obj(m[k, 1])} for k in range(3)], "gadget": gadget}

    want = {"params": {"ring_dim": N, "q": QC, "crt_moduli": list(Q), "p": 1 << 16, "sigma": 6.4,
                       "gadget_base": 1 << 20, "gadget_len": 3, "security_level": "Bits128"},
            "k_g": ksm_obj(k_g), "k_h": ksm_obj(k_h), "galois_keys": [ksm_obj(g) for g in galois],
            "rgsw_gadget": gadget, "crs_a_vectors": [[int(x) for x in v] for v in crs_a],
            "packing_k_g": ksm_obj(pk_g), "packing_k_h": None,
            "inspiring_precomp": {"a_hat": poly_obj(a_hat),
                                  "bold_t": [[poly_obj(bold_t[3 * i + k]) for k in range(3)] for i in range(15)],
                                  "bold_t_bar": [], "bold_t_hat": [], "num_to_pack": 16, "ring_dim": N, "q": QC},
            "inspiring_w_seed": list(wseed), "inspiring_v_seed": list(vseed), "inspiring_num_columns": 16}
    assert path.read_bytes() == compact(want)


def test_large_query_parallel_parse(wire):
    """Queries of 64 KB and more have their coefficient arrays located by a
    structural pass and parsed in parallel; any failure re-parses in one pass,
    so errors read as the sequential parser's.  Also: duplicate fields,
    nested arrays, and concurrent callers sharing the worker threads."""
    import threading

    inspire, w = wire
    rng = np.random.default_rng(8)
    params = inspire.InspireParams(p=1 << 16)
    seeds = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
    b_rows, y_body = rand_polys(rng, 6), rand_polys(rng, 3)
    good = compact(query_obj(5, seeds, b_rows, y_body))
    assert len(good) > 300_000
    q = w.seeded_query_from_json(params, good)
    assert np.array_equal(q.b_rows, b_rows) and np.array_equal(q.inspiring_packing_keys.y_body, y_body)
    # a bad token in the last y_body polynomial: reported at its byte offset
    key = b'"y_body":['
    start = good.index(key) + len(key)
    for _ in range(2):
        start = good.index(b'"coeffs":[', start) + len(b'"coeffs":[')
    start = good.index(b'"coeffs":[', start) + len(b'"coeffs":[')
    pos = good.index(b",", start + 5000) + 1
    bad = good[:pos] + b"x" + good[pos + 1:]
    with pytest.raises(inspire.PirError, match=f"at byte {pos}"):
        w.seeded_query_from_json(params, bad)
    # a duplicate coeffs field (serde's derive rejects it)
    dup = good.replace(b'"coeffs":', b'"coeffs":[1],"coeffs":', 1)
    with pytest.raises(inspire.PirError, match="duplicate field"):
        w.seeded_query_from_json(params, dup)
    # a nested array inside a coefficient array
    nested = good.replace(b'"coeffs":[', b'"coeffs":[[1],', 1)
    with pytest.raises(inspire.PirError):
        w.seeded_query_from_json(params, nested)
    # concurrent callers: every result exact
    bodies = []
    for k in range(8):
        br, yb = rand_polys(rng, 6), rand_polys(rng, 3)
        bodies.append((compact(query_obj(k, seeds, br, yb)), br, yb))
    errors = []

    def worker(k):
        try:
            for rep in range(5):
                body, br, yb = bodies[(k + rep) % len(bodies)]
                qq = w.seeded_query_from_json(params, body)
                assert np.array_equal(qq.b_rows, br) and np.array_equal(qq.inspiring_packing_keys.y_body, yb)
        except BaseException as e:  # reported below
            errors.append(e)

    ths = [threading.Thread(target=worker, args=(k,)) for k in range(6)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    assert not errors, errors[0]


def test_query_json_mutations_differential(wire):
    """Random single-byte mutations of a full-size SeededClientQuery (the
    parallel-parse path): the native parser accepts a body only if Python's
    json accepts it, and then returns exactly the values json reads (when the
    crate's field rules hold) -- never a silently different query."""
    inspire, w = wire
    rng = np.random.default_rng(77)
    params = inspire.InspireParams(p=1 << 16)
    seeds = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
    b_rows, y_body = rand_polys(rng, 6), rand_polys(rng, 3)
    good = compact(query_obj(9, seeds, b_rows, y_body))
    alphabet = b'0123456789,[]{}":-. eEtrufalsnx'
    accepted = 0
    for trial in range(300):
        body = bytearray(good)
        for _ in range(int(rng.integers(1, 3))):
            pos = int(rng.integers(0, len(body)))
            body[pos] = alphabet[int(rng.integers(0, len(alphabet)))]
        body = bytes(body)
        try:
            ref = json.loads(body)
        except ValueError:
            ref = None
        try:
            q = w.seeded_query_from_json(params, body)
        except inspire.PirError:
            continue
        assert ref is not None, "native parser accepted a body json rejects"
        accepted += 1
        rows = ref["rgsw_ciphertext"]["rows"]
        assert q.shard_id == ref["shard_id"]
        assert np.array_equal(q.seeds, np.array([r["seed"] for r in rows], dtype=np.uint8))
        assert np.array_equal(q.b_rows, np.array([r["b"]["coeffs"] for r in rows], dtype=np.uint64))
        keys = ref.get("inspiring_packing_keys")
        if keys is not None and keys.get("y_body"):
            assert np.array_equal(q.inspiring_packing_keys.y_body,
                                  np.array([p["coeffs"] for p in keys["y_body"]], dtype=np.uint64))
    assert accepted > 20  # mutations inside numbers that keep the residues reduced
