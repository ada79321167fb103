"""GPU tree packing (respond_one_packing / respond_seeded_packed,
src/pir/respond.rs:213-268, 428-435) through the C ABI, bit-exact against the
oracle's restatement of pack_lwes (src/inspiring/automorph_pack.rs:171-485)
with the CRS's Galois keys (src/pir/setup.rs:164-173): both automorphism
modes (compat returns the crate's b polynomial of dimension 2d), full and
seeded queries, first and partial last shard, 1, 2 and 16 columns (one LWE
is returned unpacked, automorph_pack.rs:439-446), the variant dispatch, and
the errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
W_SEED = bytes(range(40, 72))


@pytest.fixture(scope="module")
def tree(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    ctx = O.Ctx()
    client = O.Client(ctx, seed=4, rng_seed=44)
    keys = client.galois_keys()
    return dict(O=O, inspire=inspire, ctx=ctx, client=client, keys=keys, dbs={})


def world(T, mode, gamma):
    """CRS + database (2 shards, the last partial) for `gamma` columns."""
    key = (mode, gamma)
    if key not in T["dbs"]:
        inspire = T["inspire"]
        entry = 2 * gamma
        rng = np.random.default_rng(gamma)
        n_entries = N + 700
        db = rng.integers(0, 256, size=n_entries * entry, dtype=np.uint8)
        crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, gamma, mode=mode)
        crs.load_galois_keys(T["keys"])
        edb = inspire.EncodedDatabase(crs, db, entry)
        shards = [T["ctx"].encode_shard(db, entry, s) for s in range(2)]
        T["dbs"][key] = (crs, edb, db, shards)
    return T["dbs"][key]


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
@pytest.mark.parametrize("gamma,index", [(16, 5), (16, N + 699), (2, 77), (1, 1500)])
def test_seeded_packed_bit_exact(tree, mode, gamma, index):
    T = tree
    O, inspire, ctx, client = T["O"], T["inspire"], T["ctx"], T["client"]
    crs, edb, db, shards = world(T, mode, gamma)
    sid, local = divmod(index, N)
    seeds, b_rows = client.query_seeded(local)
    omode = O.MODE_CRT_FIXED if mode == "crt_fixed" else O.MODE_COMPAT
    want_a, want_b = ctx.respond_one_packing(shards[sid], ctx.expand_rgsw(seeds, b_rows), T["keys"], mode=omode)
    resp = inspire.respond_seeded_packed(crs, edb, inspire.SeededClientQuery(sid, seeds, b_rows))
    assert resp.column_ciphertexts == []
    assert np.array_equal(resp.ciphertext.a, want_a)
    assert resp.ciphertext.b.size == want_b.size
    assert np.array_equal(resp.ciphertext.b, want_b)


def test_full_query_and_variant_dispatch(tree):
    T = tree
    O, inspire, ctx, client = T["O"], T["inspire"], T["ctx"], T["client"]
    crs, edb, db, shards = world(T, "crt_fixed", 16)
    seeds, b_rows = client.query_seeded(1234)
    rgsw = ctx.expand_rgsw(seeds, b_rows)
    want_a, want_b = ctx.respond_one_packing(shards[0], rgsw, T["keys"], mode=O.MODE_CRT_FIXED)
    full = inspire.respond_one_packing(crs, edb, inspire.ClientQuery(0, rgsw.reshape(6, 2, 2 * N)))
    assert np.array_equal(full.ciphertext.a, want_a) and np.array_equal(full.ciphertext.b, want_b)
    q = inspire.SeededClientQuery(0, seeds, b_rows, packing_mode="tree")
    via = inspire.respond_seeded_with_variant(crs, edb, q, inspire.InspireVariant.OnePacking)
    assert np.array_equal(via.ciphertext.a, want_a) and np.array_equal(via.ciphertext.b, want_b)


def test_tree_errors(tree):
    T = tree
    inspire, client = T["inspire"], T["client"]
    crs, edb, db, shards = world(T, "crt_fixed", 16)
    seeds, b_rows = client.query_seeded(3)
    with pytest.raises(inspire.PirError, match="Shard 9 not found"):
        inspire.respond_seeded_packed(crs, edb, inspire.SeededClientQuery(9, seeds, b_rows))
    bare = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    edb2 = inspire.EncodedDatabase(bare, db, 32)
    with pytest.raises(inspire.PirError, match="Galois keys"):
        inspire.respond_seeded_packed(bare, edb2, inspire.SeededClientQuery(0, seeds, b_rows))
    with pytest.raises(inspire.PirError, match="log2"):
        bare.load_galois_keys(T["keys"][:10])
    bad = T["keys"].copy()
    bad[0, 0, 0] = 268369921
    with pytest.raises(inspire.PirError, match="reduced"):
        bare.load_galois_keys(bad)
    edb2.close()
    bare.close()


def test_batch_equals_single(tree):
    T = tree
    inspire, client = T["inspire"], T["client"]
    for mode in ("crt_fixed", "compat"):
        crs, edb, db, shards = world(T, mode, 16)
        idx = [(0, 17), (1, 600), (0, 2047)]
        qs = [client.query_seeded(li) for _, li in idx]
        a, b = inspire.respond_seeded_packed_batch(crs, edb, [s for s, _ in idx], np.stack([q[0] for q in qs]),
                                                   np.stack([q[1] for q in qs]))
        for k, (sid, li) in enumerate(idx):
            one = inspire.respond_seeded_packed(crs, edb, inspire.SeededClientQuery(sid, *qs[k]))
            assert np.array_equal(a[k], one.ciphertext.a) and np.array_equal(b[k], one.ciphertext.b)


def test_batch_column_split_regimes(tree):
    """The NoPacking front end splits a query's columns over CTAs when the
    batch is small (1 query: 16 CTAs of one column; 12 queries: 8 CTAs of two
    columns; 160 queries: one CTA per query).  The three regimes give the
    same tree-packed responses."""
    T = tree
    inspire, client = T["inspire"], T["client"]
    crs, edb, db, shards = world(T, "crt_fixed", 16)
    base = [client.query_seeded(li) for li in (5, 999, 2040, 64)]
    n = 160
    sids = [k % 2 for k in range(n)]
    seeds = np.stack([base[k % 4][0] for k in range(n)])
    rows = np.stack([base[k % 4][1] for k in range(n)])
    a_all, b_all = inspire.respond_seeded_packed_batch(crs, edb, sids, seeds, rows)
    a12, b12 = inspire.respond_seeded_packed_batch(crs, edb, sids[:12], seeds[:12], rows[:12])
    assert np.array_equal(a12, a_all[:12]) and np.array_equal(b12, b_all[:12])
    for k in (0, 5, 159):
        one = inspire.respond_seeded_packed(crs, edb, inspire.SeededClientQuery(sids[k], seeds[k], rows[k]))
        assert np.array_equal(one.ciphertext.a, a_all[k]) and np.array_equal(one.ciphertext.b, b_all[k])


Q = (268369921, 249561089)


def check_ks_matrix(O, ctx, kw, sk, rows, i, src):
    """rows [6][2N] of key-switching matrix i against a CPU restatement of the
    device stream: row k = (a, -a s + e + src z^k) (generate_ks_matrix,
    ks/setup.rs:118-162), a = Poly::from_seed_moduli of the first 8 words of
    block 2^52 + 3 i + k, e the Gaussian blocks 2^52 + 2^20 + (3 i + k) 256."""
    from client_stream import gaussian_blocks

    for k in range(3):
        m = 3 * i + k
        w = O.chacha20_block(kw, [(2 ** 52 + m) & 0xFFFFFFFF, (2 ** 52 + m) >> 32, 0, 0])
        a = ctx.poly_from_seed(w[:8].astype("<u4").tobytes())
        assert np.array_equal(rows[2 * k], a), (i, k)
        e = gaussian_blocks(kw, 2 ** 52 + 2 ** 20 + m * (N // 8))
        a_s = ctx.poly_mul(a, sk)
        want = np.zeros(2 * N, np.uint64)
        for r in range(2):
            q = Q[r]
            sl = slice(r * N, (r + 1) * N)
            v = (src[sl].astype(np.int64) * pow(1 << 20, k, q)) % q
            v = (v - a_s[sl].astype(np.int64)) % q
            want[sl] = ((v + e % q) % q).astype(np.uint64)
        assert np.array_equal(rows[2 * k + 1], want), (i, k)


def test_galois_keygen_device(tree):
    """Galois matrices made on the device: bit-exact against a CPU restatement
    of the stream (matrix i for t = d / 2^i + 1, row k = (a, -a s + e +
    tau_t(s) z^k), setup.rs:164-173, ks/setup.rs:118-162, 218-245), and tree
    packing with them equals the oracle's with the same keys."""
    from client_stream import gaussian_blocks

    T = tree
    torch, O, inspire, ctx = pytest.importorskip("torch"), T["O"], T["inspire"], T["ctx"]
    key = bytes(range(7, 39))
    dev = torch.device("cuda:0")
    crs, edb, db, shards = world(T, "crt_fixed", 16)
    sk = T["client"].sk
    d_sk = torch.from_numpy(sk.view(np.int64).copy()).to(dev)
    d_keys = torch.zeros((11, 6, 2 * N), dtype=torch.int64, device=dev)
    d_st = torch.full((11,), -1, dtype=torch.int32, device=dev)
    inspire.galois_keygen_device(crs, key, d_sk.data_ptr(), d_keys.data_ptr(), d_st.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert not d_st.cpu().numpy().any()
    keys = d_keys.cpu().numpy().view(np.uint64)
    kw = np.frombuffer(key, dtype="<u4")
    for i in (0, 5, 10):
        check_ks_matrix(O, ctx, kw, sk, keys[i], i, ctx.automorphism(sk, (N >> i) + 1))
    crs2 = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    crs2.load_galois_keys(keys)
    edb2 = inspire.EncodedDatabase(crs2, db, 32)
    seeds, b_rows = T["client"].query_seeded(99)
    want_a, want_b = ctx.respond_one_packing(shards[0], ctx.expand_rgsw(seeds, b_rows), keys, mode=O.MODE_CRT_FIXED)
    got = inspire.respond_seeded_packed(crs2, edb2, inspire.SeededClientQuery(0, seeds, b_rows))
    assert np.array_equal(got.ciphertext.a, want_a) and np.array_equal(got.ciphertext.b, want_b)
    edb2.close()
    crs2.close()


def test_setup_keygen_device(tree):
    """setup's public keys made on the device (setup.rs:151-200): the Galois
    matrices equal galois_keygen_device's; k_g (tau_3), k_h (tau_{2d-1}) and
    packing_k_g, packing_k_h (the LWE key of s: s[0], -s[1..], lwe/enc.rs:53-66)
    bit-exact against a CPU restatement of the stream; crs_a_vectors are
    Poly::from_seed_moduli of the stream's blocks 2^53 + v."""
    T = tree
    torch, O, inspire, ctx = pytest.importorskip("torch"), T["O"], T["inspire"], T["ctx"]
    key = bytes(range(101, 133))
    dev = torch.device("cuda:0")
    crs, edb, db, shards = world(T, "crt_fixed", 16)
    sk = T["client"].sk
    d_sk = torch.from_numpy(sk.view(np.int64).copy()).to(dev)
    stream = torch.cuda.current_stream().cuda_stream
    d_ks = torch.zeros((15, 6, 2 * N), dtype=torch.int64, device=dev)
    d_crs_a = torch.zeros((N, 2 * N), dtype=torch.int64, device=dev)
    d_st = torch.full((16,), -1, dtype=torch.int32, device=dev)
    inspire.setup_keygen_device(crs, key, d_sk.data_ptr(), d_ks.data_ptr(), d_crs_a.data_ptr(), d_st.data_ptr(),
                                stream)
    d_g = torch.zeros((11, 6, 2 * N), dtype=torch.int64, device=dev)
    d_gst = torch.full((11,), -1, dtype=torch.int32, device=dev)
    inspire.galois_keygen_device(crs, key, d_sk.data_ptr(), d_g.data_ptr(), d_gst.data_ptr(), stream)
    d_ks2 = torch.zeros((15, 6, 2 * N), dtype=torch.int64, device=dev)
    d_st2 = torch.full((16,), -1, dtype=torch.int32, device=dev)
    inspire.setup_keygen_device(crs, key, d_sk.data_ptr(), d_ks2.data_ptr(), 0, d_st2.data_ptr(), stream)
    torch.cuda.synchronize()
    assert not d_st.cpu().numpy().any() and not d_gst.cpu().numpy().any()
    assert not d_st2.cpu().numpy()[:15].any()
    ks = d_ks.cpu().numpy().view(np.uint64)
    assert np.array_equal(ks[:11], d_g.cpu().numpy().view(np.uint64))
    assert np.array_equal(ks, d_ks2.cpu().numpy().view(np.uint64))
    kw = np.frombuffer(key, dtype="<u4")
    lwe = sk.copy()
    for r in range(2):
        c = sk[r * N + 1:(r + 1) * N]
        lwe[r * N + 1:(r + 1) * N] = np.where(c == 0, 0, np.uint64(Q[r]) - c)
    sources = {11: ctx.automorphism(sk, 3), 12: ctx.automorphism(sk, 2 * N - 1), 13: lwe, 14: lwe}
    for i, src in sources.items():
        check_ks_matrix(O, ctx, kw, sk, ks[i], i, src)
    # packing_k_g and packing_k_h have the same source, different draws
    assert not np.array_equal(ks[13, 0], ks[14, 0])
    crs_a = d_crs_a.cpu().numpy().view(np.uint64)
    for v in (0, 1, 777, N - 1):
        w = O.chacha20_block(kw, [(2 ** 53 + v) & 0xFFFFFFFF, (2 ** 53 + v) >> 32, 0, 0])
        assert np.array_equal(crs_a[v], ctx.poly_from_seed(w[:8].astype("<u4").tobytes())), v
    assert len({crs_a[v].tobytes() for v in range(0, N, 97)}) == len(range(0, N, 97))
    for r in range(2):
        assert crs_a[:, r * N:(r + 1) * N].max() < Q[r]


def crs_json(keys, w_seed, num_columns, p=1 << 16):
    """serde_json of ServerCrs (pir/setup.rs:52-87) as the server's crs.json:
    the fields the Respond paths read, plus small stand-ins for the others."""
    import json

    Q = (268369921, 249561089)
    qc = Q[0] * Q[1]
    gadget = {"base": 1 << 20, "len": 3, "q": qc}

    def poly(c):
        return {"coeffs": [int(x) for x in c], "moduli": list(Q), "q": qc, "dim": N,
                "crt_q0_inv_mod_q1": pow(Q[0], Q[1] - 2, Q[1]), "is_ntt": False}

    def ksm(mat):
        return {"rows": [{"a": poly(mat[2 * k]), "b": poly(mat[2 * k + 1])} for k in range(3)], "gadget": gadget}

    obj = {"params": {"ring_dim": N, "q": qc, "crt_moduli": list(Q), "p": p, "sigma": 6.4, "gadget_base": 1 << 20,
                      "gadget_len": 3, "security_level": "Bits128"},
           "k_g": ksm(keys[0]), "k_h": ksm(keys[1]),
           "galois_keys": [ksm(m) for m in keys],
           "rgsw_gadget": gadget, "crs_a_vectors": [[1, 2, 3], [4, 5, 6]],
           "packing_k_g": None, "packing_k_h": None, "inspiring_precomp": None,
           "inspiring_w_seed": list(w_seed), "inspiring_v_seed": list(range(32)),
           "inspiring_num_columns": num_columns}
    return json.dumps(obj, separators=(",", ":")).encode()


def test_crs_json_load(tree):
    """crs.json (server.rs:255-264) loaded into a context answers like a
    context loaded field by field: InspiRING with registered keys and tree
    packing with the Galois keys."""
    T = tree
    O, inspire, ctx, client = T["O"], T["inspire"], T["ctx"], T["client"]
    crs, edb, db, shards = world(T, "crt_fixed", 16)
    params = inspire.InspireParams(p=1 << 16)
    loaded = inspire.ServerCrs.load_json(params, crs_json(T["keys"], W_SEED, 16), mode="crt_fixed")
    assert loaded.inspiring_w_seed == W_SEED and loaded.inspiring_num_columns == 16
    edb2 = inspire.EncodedDatabase(loaded, db, 32)
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    y_body, _ = client.packing_keys(pack)
    seeds, b_rows = client.query_seeded(321)
    q = inspire.SeededClientQuery(1, seeds, b_rows, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=y_body))
    a = inspire.respond_seeded_inspiring(loaded, edb2, q)
    b = inspire.respond_seeded_inspiring(crs, edb, q)
    assert np.array_equal(a.ciphertext.a, b.ciphertext.a) and np.array_equal(a.ciphertext.b, b.ciphertext.b)
    ta = inspire.respond_seeded_packed(loaded, edb2, inspire.SeededClientQuery(1, seeds, b_rows))
    tb = inspire.respond_seeded_packed(crs, edb, inspire.SeededClientQuery(1, seeds, b_rows))
    assert np.array_equal(ta.ciphertext.a, tb.ciphertext.a) and np.array_equal(ta.ciphertext.b, tb.ciphertext.b)
    with pytest.raises(inspire.PirError, match="params differ"):
        inspire.ServerCrs.load_json(params, crs_json(T["keys"], W_SEED, 16, p=65537))
    with pytest.raises(inspire.PirError, match="ServerCrs JSON"):
        inspire.ServerCrs.load_json(params, crs_json(T["keys"], W_SEED, 16)[:-2])
    edb2.close()
    loaded.close()
