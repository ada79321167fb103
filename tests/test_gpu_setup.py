"""setup's CRS on the GPU: the InspiRING offline precomputation
(ServerCrs.inspiring_precomp, src/pir/setup.rs:194-224, packing_offline
src/inspiring/inspiring2.rs:926-1041) bit-exact against the oracle in both
automorphism modes, and a crs.json made from device-generated keys that the
server's loader reads back."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
W_SEED = bytes(range(140, 172))
V_SEED = bytes(range(1, 33))
Q = (268369921, 249561089)


@pytest.fixture(scope="module")
def env(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    return dict(O=oracle_mod, inspire=inspire, torch=torch, ctx=oracle_mod.Ctx())


def _uniform(rng, k):
    a = np.zeros((k, 2 * N), np.uint64)
    a[:, :N] = rng.integers(0, Q[0], size=(k, N), dtype=np.uint64)
    a[:, N:] = rng.integers(0, Q[1], size=(k, N), dtype=np.uint64)
    return a


@pytest.mark.parametrize("gamma", [16, 4, 1])
@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_inspiring_precomp_bit_exact(env, mode, gamma):
    O, inspire, ctx = env["O"], env["inspire"], env["ctx"]
    omode = O.MODE_CRT_FIXED if mode == "crt_fixed" else O.MODE_COMPAT
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, gamma, mode=mode)
    rng = np.random.default_rng(100 + gamma)
    a = _uniform(rng, gamma)
    a_hat, bold_t = crs.inspiring_precomp(a)
    want_a_hat, want_bold_t = O.Pack(ctx, gamma, W_SEED, mode=omode).packing_offline(a)
    assert np.array_equal(a_hat, want_a_hat)
    assert bold_t.shape == want_bold_t.shape
    assert np.array_equal(bold_t, want_bold_t)
    crs.close()


def test_setup_crs_json_round_trip(env, tmp_path):
    """Every public key of setup generated on the device for a client's
    secret key, the precomputation over the first num_columns crs_a_vectors
    (setup.rs:207-217), crs.json written as the crate's setup writes it, then
    loaded as the crate's server loads it: same seed, column count, Galois
    keys (tree-packing answers equal) and crs_a_vectors count."""
    O, inspire, ctx, torch = env["O"], env["inspire"], env["ctx"], env["torch"]
    params = inspire.InspireParams(p=1 << 16)
    crs = inspire.ServerCrs(params, W_SEED, 16, mode="crt_fixed")
    client = O.Client(ctx, seed=9, rng_seed=90)
    dev = torch.device("cuda:0")
    st = torch.cuda.current_stream().cuda_stream
    d_sk = torch.from_numpy(client.sk.view(np.int64).copy()).to(dev)
    d_ks = torch.zeros((15, 6, 2 * N), dtype=torch.int64, device=dev)
    d_crs_a = torch.zeros((N, 2 * N), dtype=torch.int64, device=dev)
    d_st = torch.full((16,), -1, dtype=torch.int32, device=dev)
    inspire.setup_keygen_device(crs, bytes(range(60, 92)), d_sk.data_ptr(), d_ks.data_ptr(), d_crs_a.data_ptr(),
                                d_st.data_ptr(), st)
    torch.cuda.synchronize()
    assert not d_st.cpu().numpy().any()
    ks = d_ks.cpu().numpy().view(np.uint64).reshape(15, 3, 2, 2 * N)
    crs_a = d_crs_a.cpu().numpy().view(np.uint64)
    precomp = crs.inspiring_precomp(crs_a[:16])
    pk = O.Pack(ctx, 16, W_SEED, mode=O.MODE_CRT_FIXED)
    want = pk.packing_offline(crs_a[:16])
    assert np.array_equal(precomp[0], want[0]) and np.array_equal(precomp[1], want[1])
    path = tmp_path / "crs.json"
    inspire.write_crs_json(str(path), params, k_g=ks[11], k_h=ks[12], galois_keys=ks[:11], crs_a_vectors=crs_a,
                           inspiring_w_seed=W_SEED, inspiring_v_seed=V_SEED, inspiring_num_columns=16,
                           packing_k_g=ks[13], packing_k_h=ks[14], precomp=precomp)
    loaded = inspire.ServerCrs.load_json(params, str(path), mode="crt_fixed")
    assert loaded.inspiring_w_seed == W_SEED and loaded.inspiring_num_columns == 16
    assert loaded.crs_a_vectors_count == N
    # the precomputation as written, read back with the json module
    obj = json.loads(path.read_bytes())
    assert obj["inspiring_precomp"]["a_hat"]["coeffs"] == [int(v) for v in precomp[0]]
    assert obj["inspiring_precomp"]["bold_t"][14][2]["coeffs"] == [int(v) for v in precomp[1][44]]
    assert obj["crs_a_vectors"][777] == [int(v) for v in crs_a[777]]
    assert obj["inspiring_v_seed"] == list(V_SEED) and obj["params"]["sigma"] == 6.4
    # Galois keys loaded from the file answer tree packing like keys loaded directly
    db = np.random.default_rng(3).integers(0, 256, size=N * 32, dtype=np.uint8)
    crs.load_galois_keys(ks[:11].reshape(11, 6, 2 * N))
    e1, e2 = inspire.EncodedDatabase(crs, db, 32), inspire.EncodedDatabase(loaded, db, 32)
    seeds, b_rows = client.query_seeded(1234)
    r1 = inspire.respond_seeded_packed(crs, e1, inspire.SeededClientQuery(0, seeds, b_rows))
    r2 = inspire.respond_seeded_packed(loaded, e2, inspire.SeededClientQuery(0, seeds, b_rows))
    assert np.array_equal(r1.ciphertext.a, r2.ciphertext.a) and np.array_equal(r1.ciphertext.b, r2.ciphertext.b)
    loaded.close()
    crs.close()
