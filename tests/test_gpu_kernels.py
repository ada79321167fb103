"""GPU parity: batched NTT / inverse NTT and the general external product,
through the C ABI, bit-exact against the oracle (src/math/ntt.rs,
src/rgsw/external_product.rs semantics)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048


@pytest.fixture(scope="module")
def env(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), bytes(32), 16, mode="crt_fixed")
    ctx = oracle_mod.Ctx()
    return torch, inspire, crs, ctx


def to_dev(torch, a_u32: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a_u32, dtype=np.uint32).view(np.int32)).cuda()


def from_dev(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


def uniform_polys(rng, k, moduli):
    out = np.zeros((k, 2, N), dtype=np.uint64)
    for r, q in enumerate(moduli):
        out[:, r, :] = rng.integers(0, q, size=(k, N), dtype=np.uint64)
    return out


def test_ntt_forward_matches_reference(env):
    torch, inspire, crs, ctx = env
    rng = np.random.default_rng(4)
    polys = uniform_polys(rng, 64, crs.params.crt_moduli)
    want = ctx.ntt_forward(polys.reshape(64, -1)).reshape(64, 2, N)
    d = to_dev(torch, polys.astype(np.uint32))
    inspire.ntt_forward_device(crs, d.data_ptr(), 64, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(from_dev(d).reshape(64, 2, N).astype(np.uint64), want)


def test_ntt_inverse_matches_reference(env):
    torch, inspire, crs, ctx = env
    rng = np.random.default_rng(5)
    polys = uniform_polys(rng, 64, crs.params.crt_moduli)
    ntt = ctx.ntt_forward(polys.reshape(64, -1))
    d = to_dev(torch, ntt.astype(np.uint32))
    inspire.ntt_inverse_device(crs, d.data_ptr(), 64, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(from_dev(d).reshape(64, 2, N).astype(np.uint64), polys)


def test_ntt_known_answers(env):
    """ntt.rs:646-725: zero stays zero; X * X^(n-1) = -1 via pointwise product."""
    torch, inspire, crs, ctx = env
    q0, q1 = crs.params.crt_moduli
    polys = np.zeros((3, 2, N), dtype=np.uint32)
    polys[1, :, 1] = 1
    polys[2, :, N - 1] = 1
    d = to_dev(torch, polys)
    st = torch.cuda.current_stream().cuda_stream
    inspire.ntt_forward_device(crs, d.data_ptr(), 3, st)
    torch.cuda.synchronize()
    f = from_dev(d).reshape(3, 2, N).astype(np.uint64)
    assert not f[0].any()
    # pointwise Montgomery product (R = 2^64) of the two monomials, then inverse
    prod = np.zeros((1, 2, N), dtype=np.uint64)
    for r, q in enumerate((q0, q1)):
        rinv = pow(2 ** 64, -1, q)
        prod[0, r] = np.array([int(a) * int(b) * rinv % q for a, b in zip(f[1, r], f[2, r])], dtype=np.uint64)
    d2 = to_dev(torch, prod.astype(np.uint32))
    inspire.ntt_inverse_device(crs, d2.data_ptr(), 1, st)
    torch.cuda.synchronize()
    res = from_dev(d2).reshape(2, N)
    assert res[0, 0] == q0 - 1 and res[1, 0] == q1 - 1 and not res[:, 1:].any()


def test_ntt_roundtrip_4096_polys(env):
    """The kernel microbenchmark size (4096 polys x 2 residues): inverse(forward(x)) == x."""
    torch, inspire, crs, ctx = env
    rng = np.random.default_rng(6)
    polys = uniform_polys(rng, 4096, crs.params.crt_moduli).astype(np.uint32)
    d = to_dev(torch, polys)
    st = torch.cuda.current_stream().cuda_stream
    inspire.ntt_forward_device(crs, d.data_ptr(), 4096, st)
    torch.cuda.synchronize()
    sample = from_dev(d).reshape(4096, 2, N)[[0, 1777, 4095]].astype(np.uint64)
    want = ctx.ntt_forward(polys[[0, 1777, 4095]].astype(np.uint64).reshape(3, -1)).reshape(3, 2, N)
    assert np.array_equal(sample, want)
    inspire.ntt_inverse_device(crs, d.data_ptr(), 4096, st)
    torch.cuda.synchronize()
    assert np.array_equal(from_dev(d).reshape(4096, 2, N), polys)


def test_external_product_matches_reference(env):
    torch, inspire, crs, ctx = env
    rng = np.random.default_rng(7)
    k = 8
    cts = uniform_polys(rng, 2 * k, crs.params.crt_moduli).reshape(k, 2, 2, N)
    rgsw = uniform_polys(rng, 12 * k, crs.params.crt_moduli).reshape(k, 6, 2, 2, N)
    want = np.stack([ctx.external_product(cts[i].reshape(2, -1), rgsw[i].reshape(12, -1)) for i in range(k)])
    dct, drg = to_dev(torch, cts.astype(np.uint32)), to_dev(torch, rgsw.astype(np.uint32))
    dout = torch.zeros(k * 4 * N, dtype=torch.int32, device="cuda")
    inspire.external_product_device(crs, dct.data_ptr(), drg.data_ptr(), dout.data_ptr(), k,
                                    torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = from_dev(dout).reshape(k, 2, 2 * N).astype(np.uint64)
    assert np.array_equal(got, want.reshape(k, 2, 2 * N))


def test_external_product_rgsw_one_decrypts(env):
    """external_product.rs:256-299: RLWE(m) x RGSW(1) decrypts to m."""
    torch, inspire, crs, ctx = env
    from oracle import oracle as O

    cl = O.Client(ctx, seed=3, rng_seed=9)
    msg = ctx.from_composite(np.arange(N, dtype=np.uint64) % ctx.p)
    ct = cl.rlwe_encrypt(msg)
    one = ctx.from_composite(np.array([1] + [0] * (N - 1), dtype=np.uint64))
    rg = cl.rgsw_encrypt(one)
    dct, drg = to_dev(torch, ct.astype(np.uint32)), to_dev(torch, rg.astype(np.uint32))
    dout = torch.zeros(4 * N, dtype=torch.int32, device="cuda")
    inspire.external_product_device(crs, dct.data_ptr(), drg.data_ptr(), dout.data_ptr(), 1,
                                    torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    out = from_dev(dout).reshape(2, 2 * N).astype(np.uint64)
    assert np.array_equal(cl.decrypt(out), np.arange(N, dtype=np.uint64) % ctx.p)


def test_int8_mma_probe_exact(env):
    """The INT8 tensor-core probe (mma.sync m16n8k32 s8 -> s32) accumulates
    exactly: every accumulator equals iters * (A B), which pins the fragment
    layout the probe assumes."""
    torch, inspire, crs, ctx = env
    rng = np.random.default_rng(8)
    a = rng.integers(-128, 128, size=(16, 32), dtype=np.int8)
    b = rng.integers(-128, 128, size=(32, 8), dtype=np.int8)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros(4 * 16 * 8, dtype=torch.int32, device="cuda")
    for iters in (1, 37, 4096):
        inspire.pir.int8_mma_rate_device(crs, 3, iters, da.data_ptr(), db.data_ptr(), out.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        want = iters * (a.astype(np.int64) @ b.astype(np.int64))
        got = out.cpu().numpy().reshape(4, 16, 8)
        for c in range(4):
            assert np.array_equal(got[c], want), (iters, c)
