"""GPU client side through the C ABI: seeded query generation (query_seeded,
src/pir/query.rs:43-85, as SeededRgswCiphertext::encrypt,
src/rgsw/types.rs:233-300) and client key generation (RlweSecretKey::generate,
src/rlwe/enc.rs:14-17; ClientPackingKeys::generate's y_body,
src/inspiring/inspiring2.rs:640-660, 846-902).  Bit-exact against a CPU
restatement of the generators' streams built from the oracle's ChaCha20,
Poly::from_seed_moduli, generate_mask_from_seed, apply_automorphism and
negacyclic product; errors within the crate's tail cut with the crate's sigma;
and queries and keys generated on the device, answered by the Respond path and
extracted on the device, give back the queried entries."""
import numpy as np
import pytest
from client_stream import cdt_table, gaussian_blocks, residues

pytestmark = pytest.mark.gpu

N = 2048
ELL = 3
ENTRY = 32
SIGMA = 6.4
W_SEED = bytes(range(3, 35))
KEY = bytes(range(100, 132))
Q = (268369921, 249561089)


@pytest.fixture(scope="module")
def gen(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    ctx = O.Ctx()
    client = O.Client(ctx, seed=3, rng_seed=9)
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="crt_fixed")
    return dict(O=O, ctx=ctx, client=client, crs=crs, inspire=inspire, torch=torch)


def device_queries(G, first_query, local_idx):
    torch, inspire = G["torch"], G["inspire"]
    n = len(local_idx)
    dev = torch.device("cuda:0")
    sk = torch.from_numpy(G["client"].sk.view(np.int64).copy()).to(dev)
    idx = torch.tensor(np.asarray(local_idx, np.uint32).view(np.int32), device=dev)
    seeds = torch.zeros((n, 2 * ELL, 32), dtype=torch.uint8, device=dev)
    b_rows = torch.zeros((n, 2 * ELL, 2 * N), dtype=torch.int64, device=dev)
    status = torch.full((n,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    inspire.query_seeded_device(G["crs"], sk.data_ptr(), KEY, first_query, n, idx.data_ptr(), seeds.data_ptr(),
                                b_rows.data_ptr(), status.data_ptr(), stream)
    torch.cuda.synchronize()
    return seeds.cpu().numpy(), b_rows.cpu().numpy().view(np.uint64), status.cpu().numpy()


def expected_query(G, first_query, qi, k):
    """The device generator's output for query number first_query + qi."""
    O, ctx, sk = G["O"], G["ctx"], G["client"].sk
    key = np.frombuffer(KEY, dtype="<u4")
    Qn = first_query + qi
    m = ctx.inverse_monomial(k)
    ms = ctx.poly_mul(m, sk)
    seeds = np.zeros((2 * ELL, 32), np.uint8)
    b_rows = np.zeros((2 * ELL, 2 * N), np.uint64)
    errs = np.zeros((2 * ELL, N), np.int64)
    for row in range(2 * ELL):
        c = Qn * 16 + row
        w = O.chacha20_block(key, [c & 0xFFFFFFFF, c >> 32, 0, 0])
        seeds[row] = np.frombuffer(w[:8].astype("<u4").tobytes(), np.uint8)
        e = gaussian_blocks(key, (1 << 40) + (Qn * 2 * ELL + row) * (N // 8))
        errs[row] = e
        a = ctx.poly_from_seed(seeds[row].tobytes())
        a_s = ctx.poly_mul(a, sk)
        i = row % ELL
        msg = ms if row < ELL else m
        for r in range(2):
            q = Q[r]
            z = pow(1 << 20, i, q)
            sl = slice(r * N, (r + 1) * N)
            v = (q - a_s[sl].astype(np.int64)) % q
            v = (v + e % q) % q
            v = (v + (msg[sl].astype(np.int64) * z) % q) % q
            b_rows[row, sl] = v.astype(np.uint64)
    return seeds, b_rows, errs


@pytest.mark.parametrize("first_query", [0, 12345])
def test_query_gen_bit_exact(gen, first_query):
    idxs = [0, 1, 2047, 777]
    seeds, b_rows, status = device_queries(gen, first_query, idxs)
    assert (status == 0).all()
    for qi, k in enumerate(idxs):
        want_s, want_b, _ = expected_query(gen, first_query, qi, k)
        assert np.array_equal(seeds[qi], want_s), (qi, k)
        assert np.array_equal(b_rows[qi], want_b), (qi, k)


def test_query_gen_errors_follow_crate_distribution(gen):
    """Each row decrypts to its message plus an error (b + a s - m_row), and
    the errors lie within the tail cut with the crate's sigma."""
    ctx, sk = gen["ctx"], gen["client"].sk
    idxs = list(range(0, 2048, 256))
    seeds, b_rows, status = device_queries(gen, 99, idxs)
    assert (status == 0).all()
    cdt, T = cdt_table(SIGMA)
    errs = []
    for qi, k in enumerate(idxs):
        m = ctx.inverse_monomial(k)
        ms = ctx.poly_mul(m, sk)
        for row in range(2 * ELL):
            a = ctx.poly_from_seed(seeds[qi, row].tobytes())
            dec = (b_rows[qi, row] + ctx.poly_mul(a, sk)).astype(np.uint64)
            msg = ms if row < ELL else m
            for r in range(2):
                q = np.uint64(Q[r])
                z = np.uint64(pow(1 << 20, row % ELL, Q[r]))
                sl = slice(r * N, (r + 1) * N)
                e = (dec[sl] % q + q - (msg[sl] * z) % q) % q
                e = np.where(e > q // np.uint64(2), e.astype(np.int64) - int(q), e.astype(np.int64))
                errs.append(e)
            assert np.array_equal(errs[-1], errs[-2])  # one error, both residues
    e = np.concatenate(errs[0::2])
    assert np.abs(e).max() <= T
    var = float(np.mean(e.astype(np.float64) ** 2))
    assert abs(var / (SIGMA * SIGMA) - 1.0) < 0.05, var
    assert abs(float(e.mean())) < 0.2


def test_generated_queries_retrieve_entries(gen):
    """Queries generated on the device, answered by the batched seeded Respond,
    decrypt to the queried entries (tests/e2e_pir.rs:464-535)."""
    inspire, O, ctx, client = gen["inspire"], gen["O"], gen["ctx"], gen["client"]
    rng = np.random.default_rng(77)
    n_entries = 2 * N
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    crs = gen["crs"]
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    y_body, _ = client.packing_keys(pack)
    cid = crs.register_client(inspire.ClientPackingKeys(y_body=y_body))
    targets = [5, 2047, 2048, 4000, 1234, 3071]
    seeds, b_rows, status = device_queries(gen, 1 << 20, [t % N for t in targets])
    assert (status == 0).all()
    out = inspire.respond_seeded_batch(crs, edb, [t // N for t in targets], seeds, b_rows, [cid] * len(targets))
    for k, t in enumerate(targets):
        got = client.extract_inspiring(out[k], ENTRY)
        assert np.array_equal(got, db[t * ENTRY:(t + 1) * ENTRY]), t


def test_query_gen_rejects(gen):
    inspire = gen["inspire"]
    with pytest.raises(inspire.PirError, match="2\\^36"):
        inspire.query_seeded_device(gen["crs"], 1, KEY, (1 << 36) - 1, 2, 1, 1, 1, 1, 0)
    with pytest.raises(ValueError):
        inspire.query_seeded_device(gen["crs"], 1, KEY[:16], 0, 1, 1, 1, 1, 1, 0)


def device_keys(G, first_client, n):
    torch, inspire = G["torch"], G["inspire"]
    dev = torch.device("cuda:0")
    sk = torch.zeros((n, 2 * N), dtype=torch.int64, device=dev)
    yb = torch.zeros((n, ELL, 2 * N), dtype=torch.int64, device=dev)
    inspire.client_keygen_device(G["crs"], KEY, first_client, n, sk.data_ptr(), yb.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return sk, yb


def test_client_keygen_bit_exact(gen):
    """sk = Gaussian coefficients; y_body[k] = tau_g(s) z^k - s w_mask[k] + e_k
    with g = gen_pows[1] = 2n/gamma + 1 (inspiring2.rs:115-127, 652-654)."""
    ctx = gen["ctx"]
    key = np.frombuffer(KEY, dtype="<u4")
    sk_d, yb_d = device_keys(gen, 7, 3)
    sk_d = sk_d.cpu().numpy().view(np.uint64)
    yb_d = yb_d.cpu().numpy().view(np.uint64)
    w_mask = ctx.mask_from_seed(W_SEED, ELL)
    gen_elt = 2 * N // 16 + 1
    for i in range(3):
        base = (1 << 48) + (7 + i) * 4 * (N // 8)
        s_signed = gaussian_blocks(key, base)
        s = residues(s_signed)
        assert np.array_equal(sk_d[i], s), i
        tau = ctx.automorphism(s, gen_elt)
        for k in range(ELL):
            e = gaussian_blocks(key, base + (k + 1) * (N // 8))
            sw = ctx.poly_mul(s, w_mask[k])
            want = np.zeros(2 * N, np.uint64)
            for r in range(2):
                q = Q[r]
                sl = slice(r * N, (r + 1) * N)
                z = pow(1 << 20, k, q)
                v = (tau[sl].astype(np.int64) * z) % q
                v = (v - sw[sl].astype(np.int64)) % q
                v = (v + e % q) % q
                want[sl] = v.astype(np.uint64)
            assert np.array_equal(yb_d[i, k], want), (i, k)


def test_device_client_end_to_end(gen):
    """Every client-side step on the device: keys of three clients, their
    registered packing keys, queries under each secret key, batched Respond,
    and decrypt + extract with each client's key (no oracle involved)."""
    inspire, torch = gen["inspire"], gen["torch"]
    rng = np.random.default_rng(5)
    n_entries = 3 * N
    db = rng.integers(0, 256, size=n_entries * ENTRY, dtype=np.uint8)
    crs = gen["crs"]
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    sk, yb = device_keys(gen, 100, 3)
    ybh = yb.cpu().numpy().view(np.uint64)
    cids = [crs.register_client(inspire.ClientPackingKeys(y_body=ybh[c])) for c in range(3)]
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    targets = rng.integers(0, n_entries, size=(3, 5))
    for c in range(3):
        idx = torch.tensor((targets[c] % N).astype(np.int32), device=dev)
        seeds = torch.zeros((5, 2 * ELL, 32), dtype=torch.uint8, device=dev)
        b_rows = torch.zeros((5, 2 * ELL, 2 * N), dtype=torch.int64, device=dev)
        status = torch.full((5,), -1, dtype=torch.int32, device=dev)
        inspire.query_seeded_device(crs, sk[c].data_ptr(), KEY, 1000 * c, 5, idx.data_ptr(), seeds.data_ptr(),
                                    b_rows.data_ptr(), status.data_ptr(), stream)
        torch.cuda.synchronize()
        assert not status.cpu().numpy().any()
        out = inspire.respond_seeded_batch(crs, edb, [int(t) // N for t in targets[c]], seeds.cpu().numpy(),
                                           b_rows.cpu().numpy().view(np.uint64), [cids[c]] * 5)
        d_ct = torch.from_numpy(out.view(np.int64)).to(dev)
        ent = torch.zeros((5, ENTRY), dtype=torch.uint8, device=dev)
        inspire.pir.extract_inspiring_device(crs, sk[c].data_ptr(), d_ct.data_ptr(), 5, ENTRY, ent.data_ptr(), stream)
        torch.cuda.synchronize()
        got = ent.cpu().numpy()
        for j, t in enumerate(targets[c]):
            assert np.array_equal(got[j], db[t * ENTRY:(t + 1) * ENTRY]), (c, t)


def test_client_keygen_rejects(gen):
    inspire = gen["inspire"]
    with pytest.raises(inspire.PirError, match="2\\^30"):
        inspire.client_keygen_device(gen["crs"], KEY, (1 << 30) - 1, 2, 1, 1, 0)
