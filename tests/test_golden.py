"""Golden fixtures (tests/golden/golden.json, made by make_golden.py): the
oracle reproduces them on CPU and the GPU path reproduces them through the C
ABI."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402

GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def test_oracle_reproduces_golden(oracle_mod):
    got = MG.compute(oracle_mod)
    for key in ("ntt_forward", "poly_from_seed", "query", "respond_compat", "respond_crt_fixed"):
        assert got[key] == GOLD[key], key


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["compat", "crt_fixed"])
def test_gpu_reproduces_golden_respond(oracle_mod, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    O = oracle_mod
    ctx, db, client, seeds, b_rows = MG.inputs(O)
    pack = O.Pack(ctx, 16, MG.W_SEED, mode=O.MODE_COMPAT if mode == "compat" else O.MODE_CRT_FIXED)
    y_body, _ = client.packing_keys(pack)
    assert MG.digest(y_body) == GOLD["respond_" + mode]["y_body_sha256"]
    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), MG.W_SEED, 16, mode=mode)
    edb = inspire.EncodedDatabase(crs, db, MG.ENTRY)
    q = inspire.SeededClientQuery(0, seeds, b_rows, inspiring_packing_keys=inspire.ClientPackingKeys(y_body=y_body))
    r = inspire.respond_seeded_inspiring(crs, edb, q)
    ct = np.stack([r.ciphertext.a, r.ciphertext.b])
    assert MG.digest(ct) == GOLD["respond_" + mode]["sha256"]


@pytest.mark.gpu
def test_gpu_reproduces_golden_ntt(oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import inspire

    crs = inspire.ServerCrs(inspire.InspireParams(p=1 << 16), MG.W_SEED, 16)
    polys = MG.formula_polys(4, crs.params.crt_moduli).astype(np.uint32)
    d = torch.from_numpy(polys.view(np.int32)).cuda()
    inspire.ntt_forward_device(crs, d.data_ptr(), 4, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    out = d.cpu().numpy().view(np.uint32).astype(np.uint64).reshape(4, -1)
    assert MG.digest(out) == GOLD["ntt_forward"]["sha256"]
