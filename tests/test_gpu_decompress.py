"""GPU point decoding (helios/src/x64/helios_frombytes.cpp:59-109, selene twin)
against the reference's from_bytes golden vectors and the oracle, and MSMs
fed with 32-byte encodings."""

import numpy as np
import pytest

import oracle
from conftest import CURVES, oracle_inputs

pytestmark = pytest.mark.gpu

HS_JAC51, HS_AFF51, HS_AFF, HS_COMPRESSED = 0, 1, 2, 3


def hx(s):
    return bytes.fromhex(s)


@pytest.mark.parametrize("curve", [0, 1])
def test_golden_from_bytes(ctx, golden, curve):
    import helioselene_gb300 as hs
    name = "helios" if curve == 0 else "selene"
    cls = hs.HeliosPoint if curve == 0 else hs.SelenePoint
    for v in golden[name + "_point"]["from_bytes"]:
        P = cls.from_bytes(hx(v["input"]), ctx)
        if v["result"] in (None, "", "invalid"):
            assert P is None, v["label"]
        else:
            assert P is not None and P.to_bytes(ctx).hex() == v["result"], v["label"]


def _encodings(curve, n, seed):
    """valid encodings of random points plus invalid ones: x >= m, no square root,
    the identity's zero bytes, and both parities"""
    sc, pts, _ = oracle_inputs(curve, n, seed=seed)
    enc = oracle.compress(curve, pts).reshape(n, 32).copy()
    rng = np.random.default_rng(seed)
    m = (2**255 - 19) if curve == 0 else int(oracle_field_q())
    bad_x = [(m + k).to_bytes(32, "little") for k in (0, 1, 5)] + [(2**255 - 1).to_bytes(32, "little")]
    for j, b in enumerate(bad_x):
        enc[j] = np.frombuffer(b, np.uint8)
    enc[len(bad_x)] = 0                       # identity encoding: rejected
    enc[len(bad_x) + 1, 31] ^= 0x80           # other parity: still valid
    idx = rng.choice(np.arange(len(bad_x) + 2, n), size=n // 4, replace=False)
    enc[idx, 0] ^= rng.integers(1, 256, idx.size, dtype=np.uint8)  # random x: about half have no root
    return enc


def oracle_field_q():
    from helioselene_gb300.workload import FIELD
    return FIELD[1]


@pytest.mark.parametrize("curve", [0, 1])
def test_decompress_matches_oracle(ctx, curve):
    n = 4096
    enc = _encodings(curve, n, seed=11 + curve)
    want, nbad = oracle.decompress(curve, enc.reshape(-1))
    got, valid = ctx.decompress(curve, enc, HS_AFF, check=False)
    assert nbad > 0 and (~valid).sum() == nbad
    assert got.tobytes() == want.tobytes()
    # the reference's records: identity (1:1:0) where invalid
    got51, valid51 = ctx.decompress(curve, enc, HS_JAC51, check=False)
    assert (valid51 == valid).all()
    re = ctx.compress(curve, got51, HS_JAC51).reshape(n, 32)
    assert (re[valid] == enc[valid]).all()
    assert not re[~valid].any()


@pytest.mark.parametrize("curve", [0, 1])
def test_decompress_raises_on_invalid(ctx, curve):
    import helioselene_gb300 as hs
    with pytest.raises(hs.HsError):
        ctx.decompress(curve, bytes(32), HS_AFF)


@pytest.mark.parametrize("curve", [0, 1])
def test_msm_on_encodings(ctx, curve):
    import helioselene_gb300 as hs
    n = 3000
    sc, pts, _ = oracle_inputs(curve, n, seed=29 + curve, edge_fraction=0.02)
    nz = np.frombuffer(pts, np.uint8).reshape(n, 64).any(axis=1)
    sc, pts = sc[nz], np.frombuffer(pts, np.uint8).reshape(n, 64)[nz]   # identity has no valid encoding
    enc = oracle.compress(curve, pts.reshape(-1))
    want = oracle.msm(curve, sc, pts.reshape(-1))
    assert ctx.msm(curve, sc, enc, HS_COMPRESSED) == want
    assert ctx.msm_batch([(curve, sc, enc), (curve, sc[:100], enc[:3200])], HS_COMPRESSED)[0] == want
    bad = enc.copy().reshape(-1, 32)
    bad[7] = 0
    with pytest.raises(hs.HsError):
        ctx.msm(curve, sc, bad, HS_COMPRESSED)


@pytest.mark.parametrize("curve", [0, 1])
def test_decompress_device(ctx, curve):
    import torch
    n = 1000
    enc = _encodings(curve, n, seed=5 + curve)
    d_in = torch.from_numpy(enc.reshape(-1).copy()).cuda()
    d_out = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    d_valid = torch.empty(n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.decompress_device(curve, d_in.data_ptr(), n, d_out.data_ptr(), d_valid.data_ptr())
    torch.cuda.synchronize()
    want, nbad = oracle.decompress(curve, enc.reshape(-1))
    assert d_out.cpu().numpy().tobytes() == want.tobytes()
    assert int((d_valid.cpu().numpy() == 0).sum()) == nbad
