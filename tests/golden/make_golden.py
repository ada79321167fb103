"""Generate tests/golden/golden.json from the oracle.

The inputs are deterministic (formula-built database bytes, fixed seeds and
the oracle's seeded client), so the fixture stores SHA-256 digests of the
outputs plus a few leading values.  test_golden.py checks that the oracle still
reproduces them (CPU) and that the GPU path does (GPU).

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N = 2048
ENTRY = 32
W_SEED = bytes(range(50, 82))
QUERY_INDEX = 1500
SEED_POLY = bytes(range(1, 33))


def formula_db(n_entries, entry_size):
    i = np.arange(n_entries, dtype=np.uint64)[:, None]
    j = np.arange(entry_size, dtype=np.uint64)[None, :]
    v = (i * np.uint64(2654435761) + j * np.uint64(40503) + (i * j) % np.uint64(251)) >> np.uint64(3)
    return (v & np.uint64(0xFF)).astype(np.uint8).reshape(-1)


def formula_polys(k, moduli):
    out = np.zeros((k, 2, N), dtype=np.uint64)
    x = np.arange(k * N, dtype=np.uint64).reshape(k, N)
    for r, q in enumerate(moduli):
        out[:, r, :] = (x * np.uint64(6364136223846793005) + np.uint64(1442695040888963407 + r)) % np.uint64(q)
    return out


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def inputs(O):
    ctx = O.Ctx()
    db = formula_db(N, ENTRY)
    client = O.Client(ctx, seed=42, rng_seed=43)
    seeds, b_rows = client.query_seeded(QUERY_INDEX)
    return ctx, db, client, seeds, b_rows


def compute(O):
    ctx, db, client, seeds, b_rows = inputs(O)
    out = {}
    polys = formula_polys(4, ctx.moduli)
    fwd = ctx.ntt_forward(polys.reshape(4, -1))
    out["ntt_forward"] = {"sha256": digest(fwd), "head": [int(v) for v in fwd[0, :4]]}
    seedpoly = ctx.poly_from_seed(SEED_POLY)
    out["poly_from_seed"] = {"sha256": digest(seedpoly), "head": [int(v) for v in seedpoly[:4]],
                             "head_res1": [int(v) for v in seedpoly[N:N + 4]]}
    out["query"] = {"seeds_sha256": hashlib.sha256(seeds.tobytes()).hexdigest(), "b_rows_sha256": digest(b_rows)}
    for name, mode in (("compat", O.MODE_COMPAT), ("crt_fixed", O.MODE_CRT_FIXED)):
        # fresh client state per mode, as the GPU test builds it
        ctx, db, client, seeds, b_rows = inputs(O)
        shard = ctx.encode_shard(db, ENTRY, 0)
        rgsw = ctx.expand_rgsw(seeds, b_rows)
        pack = O.Pack(ctx, 16, W_SEED, mode=mode)
        y_body, _ = client.packing_keys(pack)
        ct = ctx.respond_inspiring(shard, rgsw, W_SEED, mode=mode, pack=pack, y_body=y_body)
        out["respond_" + name] = {"sha256": digest(ct), "a_head": [int(v) for v in ct[0, :4]],
                                  "b_head": [int(v) for v in ct[1, :4]],
                                  "y_body_sha256": digest(y_body)}
    return out


if __name__ == "__main__":
    from oracle import oracle as O

    res = compute(O)
    res["_about"] = ("SHA-256 digests of oracle outputs on deterministic inputs; generated by "
                     "tests/golden/make_golden.py")
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res, indent=1)[:400])
