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
