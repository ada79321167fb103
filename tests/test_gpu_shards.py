"""The crate's binary shard files (save_shards_binary / load_shard_binary,
src/pir/mmap.rs:19-122) loaded straight into HBM: the loaded database answers
exactly like the one built from the raw entries, the writer produces the
format byte for byte, and the loader reports missing shards and malformed
files."""
import os
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(21, 53))
Q = (268369921, 249561089)


def write_shard_file(path, shard_id, polys):
    """save_shards_binary for one shard (mmap.rs:19-53): header, then every
    polynomial's residue-major u64 coefficients, little-endian."""
    with open(path, "wb") as f:
        f.write(struct.pack("<IIII", shard_id, len(polys), N, 2))
        f.write(struct.pack("<QQ", *Q))
        for p in polys:
            f.write(np.ascontiguousarray(p, dtype="<u8").tobytes())


@pytest.fixture(scope="module")
def world(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(5)
    n_entries = 3 * N + 123  # four shards, the last one partial
    raw = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    ctx = O.Ctx()
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    client = O.Client(ctx, seed=4, rng_seed=44)
    yb, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=yb))
    shards = [ctx.encode_shard(raw, ENTRY, s) for s in range(4)]
    return dict(O=O, inspire=inspire, ctx=ctx, crs=crs, client=client, cid=cid, raw=raw, shards=shards)


def queries(W, idxs):
    seeds = np.zeros((len(idxs), 6, 32), np.uint8)
    brows = np.zeros((len(idxs), 6, 2 * N), np.uint64)
    for k, ix in enumerate(idxs):
        seeds[k], brows[k] = W["client"].query_seeded(ix % N)
    return [ix // N for ix in idxs], seeds, brows


def test_loaded_shards_answer_like_raw(world, tmp_path):
    W = world
    inspire = W["inspire"]
    for s, polys in enumerate(W["shards"]):
        write_shard_file(tmp_path / f"shard-{s:04d}.bin", s, polys)
    loaded = inspire.EncodedDatabase.load_shards(W["crs"], tmp_path)
    direct = inspire.EncodedDatabase(W["crs"], W["raw"], ENTRY)
    assert loaded.num_shards == direct.num_shards == 4
    assert loaded.device_bytes == direct.device_bytes
    idxs = [0, 2047, 2048, 3 * N + 122, 4100]
    sids, seeds, brows = queries(W, idxs)
    a = inspire.respond_seeded_batch(W["crs"], loaded, sids, seeds, brows, [W["cid"]] * len(idxs))
    b = inspire.respond_seeded_batch(W["crs"], direct, sids, seeds, brows, [W["cid"]] * len(idxs))
    assert np.array_equal(a, b)
    for k, ix in enumerate(idxs):
        got = W["client"].extract_inspiring(a[k], ENTRY)
        assert np.array_equal(got, W["raw"][ix * ENTRY:(ix + 1) * ENTRY])


def test_saved_files_match_format(world, tmp_path):
    W = world
    inspire = W["inspire"]
    direct = inspire.EncodedDatabase(W["crs"], W["raw"], ENTRY)
    out = tmp_path / "saved"
    ref = tmp_path / "ref"
    out.mkdir()
    ref.mkdir()
    direct.save_shards(out)
    for s, polys in enumerate(W["shards"]):
        write_shard_file(ref / f"shard-{s:04d}.bin", s, polys)
    assert sorted(os.listdir(out)) == sorted(os.listdir(ref))
    for name in os.listdir(ref):
        assert (out / name).read_bytes() == (ref / name).read_bytes(), name
    again = inspire.EncodedDatabase.load_shards(W["crs"], out)
    assert again.num_shards == 4


def test_loader_errors(world, tmp_path):
    W = world
    inspire = W["inspire"]
    polys = W["shards"][0]
    # a gap in the ids: two "shard-" files, shard 1 missing
    gap = tmp_path / "gap"
    gap.mkdir()
    write_shard_file(gap / "shard-0000.bin", 0, polys)
    write_shard_file(gap / "shard-0002.bin", 2, polys)
    with pytest.raises(inspire.PirError, match="Shard 1 not found"):
        inspire.EncodedDatabase.load_shards(W["crs"], gap)
    # several bad files (read in parallel): the lowest shard id's error wins
    many = tmp_path / "many"
    many.mkdir()
    for sid in range(40):
        if sid != 5:
            write_shard_file(many / f"shard-{sid:04d}.bin", sid, polys)
    write_shard_file(many / "shard-0040.bin", 40, polys)
    with open(many / "shard-0031.bin", "r+b") as f:
        f.truncate(1000)
    with pytest.raises(inspire.PirError, match="Shard 5 not found"):
        inspire.EncodedDatabase.load_shards(W["crs"], many)
    write_shard_file(many / "shard-0005.bin", 5, polys)
    with pytest.raises(inspire.PirError, match="shard-0031.bin: truncated"):
        inspire.EncodedDatabase.load_shards(W["crs"], many)
    # other moduli
    bad = tmp_path / "moduli"
    bad.mkdir()
    with open(bad / "shard-0000.bin", "wb") as f:
        f.write(struct.pack("<IIIIQQ", 0, 16, N, 2, 12289, 40961))
    with pytest.raises(inspire.PirError, match="moduli"):
        inspire.EncodedDatabase.load_shards(W["crs"], bad)
    # a polynomial that is not an encoded 16-bit column
    notcol = tmp_path / "notcol"
    notcol.mkdir()
    p2 = polys.copy()
    p2[3][N + 5] = (int(p2[3][5]) + 1) % Q[1]  # residues disagree
    write_shard_file(notcol / "shard-0000.bin", 0, p2)
    with pytest.raises(inspire.PirError, match="not an encoded 16-bit column"):
        inspire.EncodedDatabase.load_shards(W["crs"], notcol)
    # wrong column count and truncation
    few = tmp_path / "few"
    few.mkdir()
    write_shard_file(few / "shard-0000.bin", 0, polys[:8])
    with pytest.raises(inspire.PirError, match="8 polynomials"):
        inspire.EncodedDatabase.load_shards(W["crs"], few)
    cut = tmp_path / "cut"
    cut.mkdir()
    write_shard_file(cut / "shard-0000.bin", 0, polys)
    data = (cut / "shard-0000.bin").read_bytes()
    (cut / "shard-0000.bin").write_bytes(data[:-8])
    with pytest.raises(inspire.PirError, match="truncated"):
        inspire.EncodedDatabase.load_shards(W["crs"], cut)
    # an empty directory is an empty database: every shard id is unknown
    empty = tmp_path / "empty"
    empty.mkdir()
    db = inspire.EncodedDatabase.load_shards(W["crs"], empty)
    assert db.num_shards == 0
    sids, seeds, brows = queries(W, [0])
    with pytest.raises(inspire.PirError, match="Shard 0 not found"):
        inspire.respond_seeded_batch(W["crs"], db, sids, seeds, brows, [W["cid"]])
    with pytest.raises(inspire.PirError, match="cannot open"):
        inspire.EncodedDatabase.load_shards(W["crs"], tmp_path / "nope")


def encoded_db_json(shards, entry_size, total_entries, ids=None, indent=None):
    """serde_json of EncodedDatabase (pir/setup.rs:104-120, params.rs:432-450)
    with Poly's derive (math/poly.rs:64-77): the server's encoded_db.json."""
    import json

    qc = Q[0] * Q[1]

    def poly(p):
        return {"coeffs": [int(x) for x in p], "moduli": list(Q), "q": qc, "dim": N,
                "crt_q0_inv_mod_q1": pow(Q[0], Q[1] - 2, Q[1]), "is_ntt": False}

    obj = {"shards": [{"id": (ids[s] if ids else s), "polynomials": [poly(p) for p in sh]}
                      for s, sh in enumerate(shards)],
           "config": {"shard_size_bytes": N * entry_size, "entry_size_bytes": entry_size,
                      "total_entries": total_entries}}
    return json.dumps(obj, indent=indent, separators=None if indent else (",", ":")).encode()


def test_encoded_db_json_answers_like_raw(world):
    """encoded_db.json (server.rs:292-301) loaded into HBM answers bit for
    bit like the database built from the raw entries."""
    W = world
    inspire, crs, raw = W["inspire"], W["crs"], W["raw"]
    n_entries = raw.size // ENTRY
    loaded = inspire.EncodedDatabase.load_json(crs, encoded_db_json(W["shards"], ENTRY, n_entries, indent=1))
    built = inspire.EncodedDatabase(crs, raw, ENTRY)
    assert loaded.num_shards == 4
    sids, seeds, brows = queries(W, [0, N + 5, 3 * N + 122, 2 * N + 2047])
    got = inspire.respond_seeded_batch(crs, loaded, sids, seeds, brows, [W["cid"]] * 4)
    want = inspire.respond_seeded_batch(crs, built, sids, seeds, brows, [W["cid"]] * 4)
    assert np.array_equal(got, want)
    loaded.close()
    built.close()


def test_encoded_db_json_rejects(world):
    W = world
    inspire, crs, raw = W["inspire"], W["crs"], W["raw"]
    n_entries = raw.size // ENTRY
    sh = W["shards"][:2]
    with pytest.raises(inspire.PirError, match="in order"):
        inspire.EncodedDatabase.load_json(crs, encoded_db_json(sh, ENTRY, 2 * N, ids=[1, 0]))
    bad = [sh[0].copy(), sh[1]]
    bad[0][3, N + 7] = (int(bad[0][3, 7]) + 1) % Q[1]  # residues of one coefficient disagree
    with pytest.raises(inspire.PirError, match="encoded 16-bit column"):
        inspire.EncodedDatabase.load_json(crs, encoded_db_json(bad, ENTRY, 2 * N))
    with pytest.raises(inspire.PirError, match="polynomials"):
        inspire.EncodedDatabase.load_json(crs, encoded_db_json([sh[0][:15]], ENTRY, N))
    with pytest.raises(inspire.PirError, match="num_columns"):
        inspire.EncodedDatabase.load_json(crs, encoded_db_json(sh, 8, 2 * N))
    with pytest.raises(inspire.PirError, match="capacity"):
        inspire.EncodedDatabase.load_json(crs, encoded_db_json(sh, ENTRY, 2 * N + 1))
    with pytest.raises(inspire.PirError, match="EncodedDatabase JSON"):
        inspire.EncodedDatabase.load_json(crs, encoded_db_json(sh, ENTRY, 2 * N)[:-3])
