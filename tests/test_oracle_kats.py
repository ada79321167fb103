"""The oracle pinned against the reference crate's own known-answer tests.

Each test restates one test of igor53627/inspire-rs (file:line in its
docstring) and runs it on the oracle; together they pin the oracle's NTT,
polynomial algebra, gadget decomposition, external product, Galois
automorphisms, InspiRING parameters and the end-to-end InspiRING protocol.
The ChaCha20 block is pinned by RFC 8439's known-answer blocks.
"""
import numpy as np
import pytest

DEFAULT_Q = 1152921504606830593  # src/math/mod_q.rs:37


def single(O, n):
    return O.Ctx(n=n, moduli=(DEFAULT_Q,), p=65536)


# ---------------------------------------------------------------- NTT
@pytest.mark.parametrize("n,mul", [(16, 1), (1024, 1), (2048, 1000), (4096, 12345)])
def test_ntt_roundtrip(oracle_mod, n, mul):
    """ntt.rs:590-644"""
    c = single(oracle_mod, n)
    a = (np.arange(n, dtype=object) * mul % DEFAULT_Q).astype(np.uint64)
    assert np.array_equal(c.ntt_inverse(c.ntt_forward(a)), a)


def test_ntt_zero_and_constant(oracle_mod):
    """ntt.rs:646-673"""
    c = single(oracle_mod, 256)
    z = np.zeros(256, dtype=np.uint64)
    assert not c.ntt_forward(z).any()
    k = z.copy()
    k[0] = 42
    assert np.array_equal(c.ntt_inverse(c.ntt_forward(k)), k)


def test_pointwise_and_negacyclic(oracle_mod):
    """ntt.rs:675-725: 1*1 = 1 and X * X^(n-1) = -1."""
    c = single(oracle_mod, 256)
    one = np.zeros(256, dtype=np.uint64)
    one[0] = 1
    assert np.array_equal(c.poly_mul(one, one), one)
    x = np.zeros(256, dtype=np.uint64)
    x[1] = 1
    y = np.zeros(256, dtype=np.uint64)
    y[255] = 1
    r = c.poly_mul(x, y)
    assert r[0] == DEFAULT_Q - 1 and not r[1:].any()


def test_ntt_linearity(oracle_mod):
    """ntt.rs:727-749"""
    c = single(oracle_mod, 256)
    a = np.arange(256, dtype=np.uint64)
    b = (np.arange(256, dtype=np.uint64) * 2) % DEFAULT_Q
    fa, fb = c.ntt_forward(a), c.ntt_forward(b)
    fs = c.ntt_forward((a + b) % DEFAULT_Q)
    assert np.array_equal(fs, ((fa.astype(object) + fb.astype(object)) % DEFAULT_Q).astype(np.uint64))


def test_ntt_crt_slot_semantics(oracle_mod):
    """Forward slot s of each CRT residue is R * a(psi^(2 brv(s) + 1)), R = 2^64."""
    c = oracle_mod.Ctx(n=16, moduli=oracle_mod.CRT_MODULI, p=65536)
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.integers(0, q, 16, dtype=np.uint64) for q in c.moduli])
    f = c.ntt_forward(a)
    for r, q in enumerate(c.moduli):
        psi = c.L.io_ctx_psi(c.h, r)
        assert pow(psi, 32, q) == 1 and pow(psi, 16, q) == q - 1
        R = pow(2, 64, q)
        for s in range(16):
            e = 2 * int(format(s, "04b")[::-1], 2) + 1
            val = sum(int(a[r * 16 + i]) * pow(psi, e * i, q) for i in range(16)) % q
            assert int(f[r * 16 + s]) == R * val % q


# ---------------------------------------------------------------- Poly
def test_poly_mul_identity_zero_assoc_distrib(oracle_mod):
    """poly.rs:951-1074 on the d=2048 CRT parameters."""
    O = oracle_mod
    c = O.Ctx()
    rng = np.random.default_rng(1)

    def rnd():
        return np.concatenate([rng.integers(0, q, c.n, dtype=np.uint64) for q in c.moduli])

    a, b, d = rnd(), rnd(), rnd()
    one = c.from_composite(np.array([1] + [0] * (c.n - 1), dtype=np.uint64))
    assert np.array_equal(c.poly_mul(a, one), a)
    assert not c.poly_mul(a, c.zeros()).any()
    assert np.array_equal(c.poly_mul(c.poly_mul(a, b), d), c.poly_mul(a, c.poly_mul(b, d)))
    assert np.array_equal(c.poly_mul(a, b), c.poly_mul(b, a))
    qv = np.repeat(np.array(c.moduli, dtype=object), c.n)
    bd = ((b.astype(object) + d.astype(object)) % qv).astype(np.uint64)
    lhs = c.poly_mul(a, bd)
    rhs = ((c.poly_mul(a, b).astype(object) + c.poly_mul(a, d).astype(object)) % qv).astype(np.uint64)
    assert np.array_equal(lhs, rhs)


# ---------------------------------------------------------------- gadget
def test_gadget_decompose_reconstruct(oracle_mod):
    """external_product.rs:171-220 (d=2048 CRT)."""
    O = oracle_mod
    c = O.Ctx()
    rng = np.random.default_rng(2)
    a = np.concatenate([rng.integers(0, q, c.n, dtype=np.uint64) for q in c.moduli])
    dig = c.gadget_decompose(a)
    assert np.array_equal(c.gadget_reconstruct(dig), a)
    comp = np.array([c.composite(d) for d in dig], dtype=object)
    assert (comp < (1 << 20)).all()
    assert not c.gadget_decompose(c.zeros()).any()


# ---------------------------------------------------------------- external product
@pytest.mark.parametrize("case", ["zero", "one", "three", "monomial"])
def test_external_product_kats(oracle_mod, case):
    """external_product.rs:222-365 with secure_128_d2048 (p = 65537)."""
    O = oracle_mod
    c = O.Ctx(p=65537)
    cl = O.Client(c, seed=0, rng_seed=3)
    n = c.n
    if case == "monomial":
        m = np.zeros(n, dtype=np.uint64)
        m[0] = 5
    elif case == "three":
        m = (np.arange(n) % 10).astype(np.uint64)
    else:
        m = (np.arange(n) % 65537).astype(np.uint64)
    ct = cl.rlwe_encrypt(c.from_composite(m))
    g = np.zeros(n, dtype=np.uint64)
    if case == "one":
        g[0] = 1
    elif case == "three":
        g[0] = 3
    elif case == "monomial":
        g[1] = 1
    rg = cl.rgsw_encrypt(c.from_composite(g))
    dec = cl.decrypt(c.external_product(ct, rg))
    if case == "zero":
        assert not dec.any()
    elif case == "one":
        assert np.array_equal(dec, m)
    elif case == "three":
        assert np.array_equal(dec, (m * 3) % 65537)
    else:
        exp = np.zeros(n, dtype=np.uint64)
        exp[1] = 5
        assert np.array_equal(dec, exp)


# ---------------------------------------------------------------- galois
def test_automorphism_identity_composition_inverse(oracle_mod):
    """galois.rs:182-300"""
    O = oracle_mod
    c = O.Ctx()
    rng = np.random.default_rng(4)
    a = np.concatenate([rng.integers(0, q, c.n, dtype=np.uint64) for q in c.moduli])
    assert np.array_equal(c.automorphism(a, 1), a)
    t1, t2, two_n = 3, 5, 2 * c.n
    assert np.array_equal(c.automorphism(c.automorphism(a, t2), t1), c.automorphism(a, (t1 * t2) % two_n))
    inv3 = pow(3, -1, two_n)
    assert np.array_equal(c.automorphism(c.automorphism(a, 3), inv3), a)
    # tau_{2n-1}(X) = X^{-1} = -X^{n-1}
    x = c.from_composite(np.array([0, 1] + [0] * (c.n - 2), dtype=np.uint64))
    y = c.automorphism(x, two_n - 1)
    comp = c.composite(y)
    assert comp[c.n - 1] == c.q - 1 and sum(1 for v in comp if v) == 1


# ---------------------------------------------------------------- InspiRING params
def test_pack_params_generator_and_powers(oracle_mod):
    """inspiring2.rs:1689-1742 (ring_dim 256, q = 2^60 - 2^14 + 1)."""
    O = oracle_mod
    c = single(O, 256)
    assert O.Pack(c, 8, bytes(32)).generator == 65
    p16 = O.Pack(c, 16, bytes(32))
    assert p16.generator == 33
    assert O.Pack(c, 256, bytes(32)).generator == 5
    gp = p16.gen_pows()
    assert gp[0] == 1 and gp[1] == 33
    assert all(gp[i] == pow(33, i, 512) for i in range(10))
    assert (16 * p16.mod_inv_gamma) % DEFAULT_Q == 1
    assert (8 * O.Pack(c, 8, bytes(32)).mod_inv_gamma) % DEFAULT_Q == 1


def test_automorph_tables_closed_form_equals_brute_force(oracle_mod):
    """The closed-form NTT-domain automorphism table equals the crate's
    brute-force search (inspiring2.rs:208-263) for every odd t at n=256 and
    for sampled t at n=2048 with the CRT moduli."""
    O = oracle_mod
    c = single(O, 256)
    rng = O.Rng(u64=5)
    for t in range(1, 512, 2):
        assert np.array_equal(O.automorph_table_brute(c, t, rng), O.automorph_table_closed(256, t))
    c2 = O.Ctx()
    for t in (1, 3, 257, 4095, 2049):
        assert np.array_equal(O.automorph_table_brute(c2, t, rng), O.automorph_table_closed(2048, t))


def test_faithful_pack_params_equal_hoisted(oracle_mod):
    """PackParams::new with brute-force tables and transformed monomials gives
    the same packed response as the closed forms (n=256)."""
    O = oracle_mod
    c = single(O, 256)
    rng = np.random.default_rng(6)
    db = rng.integers(0, 256, size=256 * 8, dtype=np.uint8)
    cl = O.Client(c, seed=1, rng_seed=2)
    w = bytes(range(32))
    pk = O.Pack(c, 4, w, mode=O.MODE_COMPAT)
    seeds, brows = cl.query_seeded(17)
    rg = c.expand_rgsw(seeds, brows)
    yb, _ = cl.packing_keys(pk)
    shard = c.encode_shard(db, 8, 0)
    hoisted = c.respond_inspiring(shard, rg, w, mode=O.MODE_COMPAT, pack=pk, y_body=yb)
    faithful = c.respond_inspiring(shard, rg, w, mode=O.MODE_COMPAT, pack=None, y_body=yb)
    assert np.array_equal(hoisted, faithful)


# ---------------------------------------------------------------- encode_db
def test_inverse_monomial_and_rotation(oracle_mod):
    """encode_db.rs:318-368"""
    O = oracle_mod
    c = O.Ctx()
    m0 = c.composite(c.inverse_monomial(0))
    assert m0[0] == 1 and sum(1 for v in m0 if v) == 1
    m1 = c.composite(c.inverse_monomial(1))
    assert m1[c.n - 1] == c.q - 1 and sum(1 for v in m1 if v) == 1
    h = c.from_composite(np.arange(c.n, dtype=np.uint64) + 7)
    for k in (0, 1, 100, 2047):
        r = c.composite(c.poly_mul(h, c.inverse_monomial(k)))
        assert r[0] == k + 7


def test_encode_shard_columns(oracle_mod):
    """encode_db.rs:106-181: 16-bit little-endian columns; odd entry sizes."""
    O = oracle_mod
    c = O.Ctx()
    db = np.arange(2100 * 3, dtype=np.uint64).astype(np.uint8)
    s1 = c.encode_shard(db, 3, 1)  # entries 2048..2099, 2 columns
    assert s1.shape[0] == 2
    e = 2048
    assert int(s1[0][0]) == int(db[e * 3]) | (int(db[e * 3 + 1]) << 8)
    assert int(s1[1][0]) == int(db[e * 3 + 2])
    assert not s1[:, 52:c.n].any()


# ---------------------------------------------------------------- ChaCha / rand
def test_chacha20_rfc8439_blocks(oracle_mod):
    O = oracle_mod
    zero = O.chacha20_block([0] * 8, [0, 0, 0, 0])
    assert "".join(int(w).to_bytes(4, "little").hex() for w in zero).startswith(
        "76b8e0ada0f13d90405d6ae55386bd28bdd219b8a08ded1aa836efcc8b770dc7")
    key = [int.from_bytes(bytes(range(4 * i, 4 * i + 4)), "little") for i in range(8)]
    nonce = bytes.fromhex("000000090000004a00000000")
    blk = O.chacha20_block(key, [1] + [int.from_bytes(nonce[4 * i:4 * i + 4], "little") for i in range(3)])
    assert [int(x) for x in blk[:4]] == [0xE4E7F110, 0x15593BD1, 0x1FDD0F50, 0xC47120A3]


def test_rng_stream_order_and_range(oracle_mod):
    O = oracle_mod
    r1, r2 = O.Rng(seed=bytes(32)), O.Rng(seed=bytes(32))
    lo, hi = r1.next_u32(), r1.next_u32()
    assert r2.next_u64() == lo | (hi << 32)
    assert lo == 0xADE0B876  # first keystream word of the all-zero key
    c = O.Ctx()
    p = c.poly_from_seed(bytes(range(32)))
    assert (p[:c.n] < c.moduli[0]).all() and (p[c.n:] < c.moduli[1]).all()
    assert np.array_equal(p, c.poly_from_seed(bytes(range(32))))


# ---------------------------------------------------------------- end to end
@pytest.mark.parametrize("entry_size", [2, 32])
def test_e2e_inspiring_single_modulus(oracle_mod, entry_size):
    """tests/e2e_pir.rs:464-535: InspiRING packing recovers entries 0, 1, 42,
    100 with d=256, q=2^60-2^14+1, p=2^16 (the crate's own behaviour)."""
    O = oracle_mod
    c = single(O, 256)
    db = np.array([(i % 256) if j == 0 else 0 for i in range(256) for j in range(entry_size)], dtype=np.uint8)
    cl = O.Client(c, seed=0, rng_seed=1)
    w = bytes(range(32))
    gamma = max(1, (entry_size * 8 + 15) // 16)
    pk = O.Pack(c, gamma, w, mode=O.MODE_COMPAT)
    shard = c.encode_shard(db, entry_size, 0)
    for idx in (0, 1, 42, 100):
        seeds, brows = cl.query_seeded(idx)
        yb, _ = cl.packing_keys(pk)
        ct = c.respond_inspiring(shard, c.expand_rgsw(seeds, brows), w, mode=O.MODE_COMPAT, pack=pk, y_body=yb)
        assert np.array_equal(cl.extract_inspiring(ct, entry_size), db[idx * entry_size:(idx + 1) * entry_size])


def test_crt_defect_finding(oracle_mod):
    """With the two CRT moduli the crate's NTT-domain automorphism
    (inspiring2.rs:279-296) corrupts residue 1: compat responses do not
    decrypt, crt_fixed responses do."""
    O = oracle_mod
    c = O.Ctx()
    rng = np.random.default_rng(8)
    db = rng.integers(0, 256, size=2048 * 32, dtype=np.uint8)
    cl = O.Client(c, seed=0, rng_seed=9)
    w = bytes(range(32))
    shard = c.encode_shard(db, 32, 0)
    seeds, brows = cl.query_seeded(1234)
    rg = c.expand_rgsw(seeds, brows)
    ok = {}
    for mode in (O.MODE_COMPAT, O.MODE_CRT_FIXED):
        pk = O.Pack(c, 16, w, mode=mode)
        yb, _ = cl.packing_keys(pk)
        ct = c.respond_inspiring(shard, rg, w, mode=mode, pack=pk, y_body=yb)
        ok[mode] = np.array_equal(cl.extract_inspiring(ct, 32), db[1234 * 32:1235 * 32])
    assert ok[O.MODE_CRT_FIXED] and not ok[O.MODE_COMPAT]


def test_respond_nopacking_extracts(oracle_mod):
    """respond (NoPacking, respond.rs:71-115): every column ciphertext decrypts
    to its entry value at coefficient 0 (tests/e2e_pir.rs:288-335)."""
    O = oracle_mod
    c = O.Ctx()
    rng = np.random.default_rng(10)
    db = rng.integers(0, 256, size=2048 * 4, dtype=np.uint8)
    cl = O.Client(c, seed=0, rng_seed=11)
    seeds, brows = cl.query_seeded(99)
    _, cols = c.respond_nopacking(c.encode_shard(db, 4, 0), c.expand_rgsw(seeds, brows), with_columns=True)
    vals = [int(cl.decrypt(col.reshape(-1))[0]) for col in cols]
    ent = db[99 * 4:100 * 4]
    assert vals == [int(ent[0]) | (int(ent[1]) << 8), int(ent[2]) | (int(ent[3]) << 8)]


# ---------------------------------------------------------------- tree packing
def _lwe_leaves(O, c, cl, msgs, trivial=False):
    """RLWE encryptions of m at coefficient 0, as pack_lwes sees their
    sample_extract_coeff0 LWEs: leaf a = the RLWE a, b = b.coeff(0)
    (automorph_pack.rs:349-405); trivial LWEs have a = 0, b = delta * m."""
    la, bv = [], []
    for m in msgs:
        if trivial:
            la.append(c.zeros())
            bv.append((int(c.delta) * m) % int(c.q))
            continue
        msg = c.zeros()
        msg[0] = m
        if c.crt == 2:
            msg[c.n] = m
        ct = cl.rlwe_encrypt(msg)
        la.append(ct[0])
        bv.append(c.L.io_poly_coeff(c.h, np.ascontiguousarray(ct[1]), 0))
    return np.stack(la), np.array(bv, dtype=np.uint64)


@pytest.mark.parametrize("case", ["single", "two", "trivial", "multiple"])
def test_pack_lwes_kats(oracle_mod, case):
    """automorph_pack.rs tests test_pack_lwes_single / _two / _trivial /
    _multiple (d = 256, q = 2^60 - 2^14 + 1, p = 2^16): coefficient i of
    the packed decryption is m_i * d mod p (m itself for a single LWE)."""
    O = oracle_mod
    c = single(O, 256)
    cl = O.Client(c, seed=0, rng_seed=21)
    keys = cl.galois_keys()
    msgs = {"single": [12345], "two": [100, 200], "trivial": [100, 200, 300, 400],
            "multiple": [100, 200, 300, 400]}[case]
    la, bv = _lwe_leaves(O, c, cl, msgs, trivial=case == "trivial")
    a, b = c.pack_lwes(la, bv, keys, mode=O.MODE_COMPAT)
    dec = cl.decrypt(np.stack([a, b]))
    if case == "single":
        assert int(dec[0]) == 12345
    else:
        for i, m in enumerate(msgs):
            assert int(dec[i]) == (m * 256) % 65536


def test_tree_packing_crt_default_params_finding(oracle_mod):
    """respond_one_packing at d = 2048 with the two CRT moduli and the crate's
    default p = 65537 (params.rs:213-230) does not give decryptable responses:
    (1) the crate's last step (automorph_pack.rs:474-484) returns a b
    polynomial of dimension 2d; (2) even with the b values added per
    composite coefficient, the 11 levels of key switching leave noise above
    delta / 2, so extract_packed (extract.rs:113-148) loses columns."""
    O = oracle_mod
    c = O.Ctx(p=65537)
    rng = np.random.default_rng(12)
    db = rng.integers(0, 256, size=2048 * 32, dtype=np.uint8)
    cl = O.Client(c, seed=3, rng_seed=13)
    keys = cl.galois_keys()
    shard = c.encode_shard(db, 32, 0)
    seeds, brows = cl.query_seeded(5)
    rg = c.expand_rgsw(seeds, brows)
    a_f, b_f = c.respond_one_packing(shard, rg, keys, mode=O.MODE_CRT_FIXED)
    a_c, b_c = c.respond_one_packing(shard, rg, keys, mode=O.MODE_COMPAT)
    assert b_f.size == c.plen and b_c.size == 2 * c.plen and np.array_equal(a_c, a_f)
    assert np.array_equal(b_c[16:c.n], b_f[16:c.n])  # residue-0 words without an added b value
    got = cl.extract_packed(np.stack([a_f, b_f]), 32)
    ent = db[5 * 32:6 * 32]
    # a column is lost exactly when its coefficient's noise exceeds delta / 2
    t = np.zeros(c.plen, np.uint64)
    c.L.io_poly_mul(c.h, np.ascontiguousarray(a_f), np.ascontiguousarray(cl.sk), t)
    q, D = int(c.q), int(c.delta)
    lost, over = [], []
    for k in range(16):
        v = (int(c.L.io_poly_coeff(c.h, t, k)) + int(c.L.io_poly_coeff(c.h, np.ascontiguousarray(b_f), k))) % q
        m = int(ent[2 * k]) | (int(ent[2 * k + 1]) << 8)
        err = (v - D * ((m * 2048) % 65537)) % q
        if min(err, q - err) > D // 2:
            over.append(k)
        if (got[2 * k], got[2 * k + 1]) != (ent[2 * k], ent[2 * k + 1]):
            lost.append(k)
    assert over and lost == over
