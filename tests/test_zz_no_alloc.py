"""The allocation-free tree-packing entry (static device scratch, device
buffers) against the allocating one (inspire_respond_seeded_packed), on two
calls in a row that reuse the same scratch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
W_SEED = bytes(range(50, 82))


def test_noalloc_tree_equals_respond_seeded_packed(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    ctx = O.Ctx()
    client = O.Client(ctx, seed=6, rng_seed=66)
    rng = np.random.default_rng(66)
    db = rng.integers(0, 256, size=(2 * N + 300) * 32, dtype=np.uint8)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    for mode in ("crt_fixed", "compat"):
        crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), W_SEED, 16, mode=mode)
        crs.load_galois_keys(client.galois_keys())
        edb = inspire.EncodedDatabase(crs, db, 32)
        for call, targets in enumerate(([5, N + 17], [2 * N + 299])):
            qs = [client.query_seeded(t % N) for t in targets]
            sids = [t // N for t in targets]
            n = len(targets)
            d_sid = torch.tensor(sids, dtype=torch.int32, device=dev)
            d_seeds = torch.from_numpy(np.stack([q[0][3:6] for q in qs])).to(dev)
            d_brows = torch.from_numpy(np.stack([q[1][3:6] for q in qs]).view(np.int64)).to(dev)
            d_a = torch.zeros((n, 2 * N), dtype=torch.int64, device=dev)
            d_b = torch.zeros((n, 4 * N), dtype=torch.int64, device=dev)
            d_st = torch.full((n,), -1, dtype=torch.int32, device=dev)
            words = inspire.pir.respond_seeded_packed_noalloc_device(
                crs, edb, n, d_sid.data_ptr(), d_seeds.data_ptr(), d_brows.data_ptr(), d_a.data_ptr(),
                d_b.data_ptr(), d_st.data_ptr(), stream)
            torch.cuda.synchronize()
            assert not d_st.cpu().numpy().any()
            a = d_a.cpu().numpy().view(np.uint64)
            b = d_b.cpu().numpy().view(np.uint64)
            for k, (sid, q) in enumerate(zip(sids, qs)):
                want = inspire.respond_seeded_packed(crs, edb, inspire.SeededClientQuery(sid, *q))
                assert words == want.ciphertext.b.size, (mode, call)
                assert np.array_equal(a[k], want.ciphertext.a), (mode, call, k)
                assert np.array_equal(b[k, :words], want.ciphertext.b), (mode, call, k)
        with pytest.raises(inspire.PirError, match="at most 2"):
            inspire.pir.respond_seeded_packed_noalloc_device(crs, edb, 3, 1, 1, 1, 1, 1, 1, stream)
        edb.close()
        crs.close()
