"""The benchmark configurations at their full sizes, bit for bit against the
oracle (src/pir/respond.rs:284-398, src/math/ntt.rs:223-379,
src/rgsw/external_product.rs:88-150):

* 2^24 entries x 32 B (8192 shards, 512 MiB raw, the batched-throughput
  database): batches of B = 1, 8, 32 and 128 seeded queries per launch, in
  both automorphism modes, shard ids 0, 4095 and 8191 among random ones,
  every response of every batch compared with the oracle (shard offsets in
  the resident contracted form pass 2^32 bytes above shard 699);
* the kernel microbenchmark at its full size: all 4096 polynomials of the
  NTT and inverse-NTT batch and all 1024 external products;
* the 1024-entry CPU-runnable configuration in compat mode (its crt_fixed
  case is in test_gpu_configs.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
ENTRY = 32
W_SEED = bytes(range(90, 122))
LOG2_ENTRIES = 24


@pytest.fixture(scope="module")
def big(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    rng = np.random.default_rng(240)
    n_entries = 1 << LOG2_ENTRIES
    db = np.frombuffer(rng.bytes(n_entries * ENTRY), dtype=np.uint8)
    ctx = O.Ctx()
    clients = [O.Client(ctx, seed=40 + s, rng_seed=400 + s) for s in range(4)]
    return dict(O=O, inspire=inspire, torch=torch, ctx=ctx, db=db, n_entries=n_entries, clients=clients, rng=rng)


def _batch_queries(W, B, forced):
    """B queries: the forced shard ids first, then uniform ones; local
    indices uniform; clients in turn."""
    rng = W["rng"]
    nsh = W["n_entries"] // N
    sids = list(forced[:B]) + [int(s) for s in rng.integers(0, nsh, size=max(0, B - len(forced)))]
    locs = [int(v) for v in rng.integers(0, N, size=B)]
    cl = [k % len(W["clients"]) for k in range(B)]
    seeds = np.zeros((B, 6, 32), np.uint8)
    brows = np.zeros((B, 6, 2 * N), np.uint64)
    for k in range(B):
        seeds[k], brows[k] = W["clients"][cl[k]].query_seeded(locs[k])
    return sids, locs, cl, seeds, brows


@pytest.mark.parametrize("mode", ["crt_fixed", "compat"])
def test_batched_2p24_entries_every_response_bit_exact(big, mode):
    W = big
    O, inspire, ctx, torch = W["O"], W["inspire"], W["ctx"], W["torch"]
    omode = O.MODE_CRT_FIXED if mode == "crt_fixed" else O.MODE_COMPAT
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode=mode)
    edb = inspire.EncodedDatabase(crs, W["db"], ENTRY)
    assert edb.num_shards == 8192
    pack = O.Pack(ctx, 16, W_SEED, mode=omode)
    ybodies = [c.packing_keys(pack)[0] for c in W["clients"]]
    ids = [crs.register_client(inspire.ClientPackingKeys(y_body=yb)) for yb in ybodies]
    shard_cache = {}

    def oracle(sid, seeds, brows, c):
        if sid not in shard_cache:
            shard_cache[sid] = ctx.encode_shard(W["db"], ENTRY, sid)
        return ctx.respond_inspiring(shard_cache[sid], ctx.expand_rgsw(seeds, brows), W_SEED, mode=omode, pack=pack,
                                     y_body=ybodies[c])

    forced = [0, 4095, 8191, 700, 8190]
    for B in (1, 8, 32, 128):
        sids, locs, cl, seeds, brows = _batch_queries(W, B, forced)
        out = inspire.respond_seeded_batch(crs, edb, sids, seeds, brows, [ids[c] for c in cl])
        for k in range(B):
            want = oracle(sids[k], seeds[k], brows[k], cl[k])
            assert np.array_equal(out[k], want), (mode, B, k, sids[k])
            if mode == "crt_fixed":
                ix = sids[k] * N + locs[k]
                got = W["clients"][cl[k]].extract_inspiring(out[k], ENTRY)
                assert np.array_equal(got, W["db"][ix * ENTRY:(ix + 1) * ENTRY]), (B, k)
    # the device-buffer batch call the throughput figure uses (b-side launch
    # + Respond launch on a caller stream), B = 128, every response
    B = 128
    sids, locs, cl, seeds, brows = _batch_queries(W, B, forced[::-1])
    dev = torch.device("cuda", 0)
    d_sid = torch.tensor(sids, dtype=torch.int32, device=dev)
    d_cid = torch.tensor([ids[c] for c in cl], dtype=torch.int32, device=dev)
    d_seeds = torch.from_numpy(np.ascontiguousarray(seeds[:, 3:6])).to(dev)
    d_brows = torch.from_numpy(np.ascontiguousarray(brows[:, 3:6]).view(np.int64)).to(dev)
    d_out = torch.zeros((B, 4 * N), dtype=torch.int64, device=dev)
    d_st = torch.full((B,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    inspire.pir.respond_seeded_batch_device(crs, edb, B, d_sid.data_ptr(), d_seeds.data_ptr(), d_brows.data_ptr(),
                                            d_cid.data_ptr(), d_out.data_ptr(), d_st.data_ptr(), stream)
    torch.cuda.synchronize()
    assert not d_st.cpu().numpy().any()
    got = d_out.cpu().numpy().view(np.uint64).reshape(B, 2, 2 * N)
    for k in range(B):
        assert np.array_equal(got[k], oracle(sids[k], seeds[k], brows[k], cl[k])), (mode, "device call", k)
    # a small batch on both Respond kernels: the two-CTA cluster kernel (the
    # default up to pair_threshold queries) and one CTA per query
    B = 8
    sids, locs, cl, seeds, brows = _batch_queries(W, B, forced[::-1])
    pair = inspire.respond_seeded_batch(crs, edb, sids, seeds, brows, [ids[c] for c in cl])
    old_threshold = crs.pair_threshold
    crs.pair_threshold = 0
    one = inspire.respond_seeded_batch(crs, edb, sids, seeds, brows, [ids[c] for c in cl])
    crs.pair_threshold = old_threshold
    assert np.array_equal(pair, one), (mode, "pair vs one CTA")
    for k in range(B):
        assert np.array_equal(pair[k], oracle(sids[k], seeds[k], brows[k], cl[k])), (mode, "pair", k)
    # all queries on one shard (the same-shard variant of the batch)
    B = 32
    sids, locs, cl, seeds, brows = _batch_queries(W, B, [8191] * B)
    out = inspire.respond_seeded_batch(crs, edb, sids, seeds, brows, [ids[c] for c in cl])
    for k in range(B):
        assert np.array_equal(out[k], oracle(8191, seeds[k], brows[k], cl[k])), (mode, "same shard", k)
    for i in ids:
        crs.release_client(i)
    edb.close()
    crs.close()


def _uniform_polys(rng, k, moduli):
    out = np.zeros((k, 2, N), dtype=np.uint64)
    for r, q in enumerate(moduli):
        out[:, r, :] = rng.integers(0, q, size=(k, N), dtype=np.uint64)
    return out


def test_kernel_microbench_full_size(big):
    """4096 polynomials x 2 residues through the batched NTT and inverse NTT,
    and 1024 external products (seeded uniform inputs), every output word
    against the oracle."""
    W = big
    inspire, ctx, torch = W["inspire"], W["ctx"], W["torch"]
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), bytes(32), 16, mode="crt_fixed")
    moduli = crs.params.crt_moduli
    dev = torch.device("cuda", 0)
    st = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(4)
    polys = _uniform_polys(rng, 4096, moduli)
    want_f = ctx.ntt_forward(polys.reshape(4096, -1)).reshape(4096, 2, N)
    d = torch.from_numpy(polys.astype(np.uint32).view(np.int32)).to(dev)
    inspire.ntt_forward_device(crs, d.data_ptr(), 4096, st)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().view(np.uint32).reshape(4096, 2, N).astype(np.uint64), want_f)
    # inverse of the reference-form values: back to the inputs, and equal to the oracle's inverse
    inspire.ntt_inverse_device(crs, d.data_ptr(), 4096, st)
    torch.cuda.synchronize()
    back = d.cpu().numpy().view(np.uint32).reshape(4096, 2, N).astype(np.uint64)
    assert np.array_equal(back, polys)
    other = _uniform_polys(rng, 4096, moduli)
    want_i = ctx.ntt_inverse(other.reshape(4096, -1)).reshape(4096, 2, N)
    d2 = torch.from_numpy(other.astype(np.uint32).view(np.int32)).to(dev)
    inspire.ntt_inverse_device(crs, d2.data_ptr(), 4096, st)
    torch.cuda.synchronize()
    assert np.array_equal(d2.cpu().numpy().view(np.uint32).reshape(4096, 2, N).astype(np.uint64), want_i)
    # 1024 external products, general RLWE (a != 0) x RGSW rows
    k = 1024
    cts = _uniform_polys(rng, 2 * k, moduli).reshape(k, 2, 2, N)
    rgsw = _uniform_polys(rng, 12 * k, moduli).reshape(k, 6, 2, 2, N)
    dct = torch.from_numpy(cts.astype(np.uint32).view(np.int32)).to(dev)
    drg = torch.from_numpy(rgsw.astype(np.uint32).view(np.int32)).to(dev)
    dout = torch.zeros(k * 4 * N, dtype=torch.int32, device=dev)
    inspire.external_product_device(crs, dct.data_ptr(), drg.data_ptr(), dout.data_ptr(), k, st)
    torch.cuda.synchronize()
    got = dout.cpu().numpy().view(np.uint32).reshape(k, 2, 2 * N).astype(np.uint64)
    for i in range(k):
        want = ctx.external_product(cts[i].reshape(2, -1), rgsw[i].reshape(12, -1))
        assert np.array_equal(got[i], want.reshape(2, 2 * N)), i
    crs.close()


def test_c1_compat_mode(big):
    """The 1024-entry configuration (InsPIRe^1 full query and InsPIRe^2
    seeded query) in compat mode, the crate's own bits."""
    W = big
    O, inspire, ctx = W["O"], W["inspire"], W["ctx"]
    db = np.random.default_rng(1).integers(0, 256, size=1024 * ENTRY, dtype=np.uint8)
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode="compat")
    edb = inspire.EncodedDatabase(crs, db, ENTRY)
    pack = O.Pack(ctx, 16, W_SEED, mode=O.MODE_COMPAT)
    client = W["clients"][0]
    y_body, _ = client.packing_keys(pack)
    keys = inspire.ClientPackingKeys(y_body=y_body)
    shard = ctx.encode_shard(db, ENTRY, 0)
    for idx in list(np.random.default_rng(2).integers(0, 1024, size=4)) + [0, 1023, 1500]:
        idx = int(idx)
        seeds, b_rows = client.query_seeded(idx)
        rgsw = ctx.expand_rgsw(seeds, b_rows)
        want = ctx.respond_inspiring(shard, rgsw, W_SEED, mode=O.MODE_COMPAT, pack=pack, y_body=y_body)
        full = inspire.respond_inspiring(crs, edb, inspire.ClientQuery(0, rgsw, inspiring_packing_keys=keys))
        seeded = inspire.respond_seeded_inspiring(crs, edb,
                                                  inspire.SeededClientQuery(0, seeds, b_rows, inspiring_packing_keys=keys))
        for r in (full, seeded):
            assert np.array_equal(np.stack([r.ciphertext.a, r.ciphertext.b]), want), idx
    edb.close()
    crs.close()
