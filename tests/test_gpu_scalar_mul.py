"""Independent variable-time scalar multiplications (helios_scalarmult_vartime,
helios/include/helios_scalarmult_vartime.h:39-57) against the reference's
scalar_mul golden vectors and the oracle."""

import numpy as np
import pytest

import oracle
from conftest import oracle_inputs

pytestmark = pytest.mark.gpu

HS_JAC51, HS_AFF51, HS_AFF, HS_COMPRESSED = 0, 1, 2, 3


def hx(s):
    return bytes.fromhex(s)


@pytest.mark.parametrize("curve", [0, 1])
def test_golden_scalar_mul(ctx, golden, curve):
    name = "helios" if curve == 0 else "selene"
    for v in golden[name + "_point"]["scalar_mul"]:
        # the identity's 32 zero bytes do not decode (from_bytes rejects them): the
        # vectors use it as the identity point, which is (0, 0) in affine form
        P, _ = oracle.decompress(curve, hx(v["point"]))
        got = ctx.scalar_mul(curve, hx(v["scalar"]), P, HS_AFF, HS_COMPRESSED)
        assert got.tobytes().hex() == v["result"], v["label"]
    enc = [v["point"] for v in golden[name + "_point"]["scalar_mul"] if any(hx(v["point"]))]
    if enc:  # decodable points also go in as encodings
        v = next(v for v in golden[name + "_point"]["scalar_mul"] if v["point"] == enc[0])
        got = ctx.scalar_mul(curve, hx(v["scalar"]), hx(v["point"]), HS_COMPRESSED, HS_COMPRESSED)
        assert got.tobytes().hex() == v["result"], v["label"]


@pytest.mark.parametrize("curve", [0, 1])
def test_scalar_mul_matches_oracle(ctx, curve):
    from helioselene_gb300.workload import ORDER, int_to_bytes32
    n = 3000
    sc, pts, _ = oracle_inputs(curve, n, seed=41 + curve)
    sc = sc.copy()
    pts = np.frombuffer(pts, np.uint8).reshape(n, 64).copy()
    sc[0] = 0
    sc[1] = int_to_bytes32(ORDER[curve] - 1)
    sc[2] = 0xFF                                   # 2^256 - 1 (unreduced)
    sc[3] = int_to_bytes32(1)
    sc[4] = int_to_bytes32(ORDER[curve])           # order: identity
    pts[5] = 0                                     # identity base
    got = ctx.scalar_mul(curve, sc, pts, HS_AFF, HS_AFF).reshape(n, 64)
    want = np.stack([np.frombuffer(oracle.scalar_mul(curve, sc[i], pts[i]), np.uint8) for i in range(n)])
    assert (got == want).all()
    assert not got[0].any() and not got[4].any() and not got[5].any()


@pytest.mark.parametrize("curve", [0, 1])
def test_scalar_mul_forms(ctx, curve):
    """reference records in and out, the drop-in signature and the point mirror"""
    import ctypes

    import helioselene_gb300 as hs
    n = 40
    sc, pts, _ = oracle_inputs(curve, n, seed=7 + curve)
    jac = hs.affine64_to_jac51(np.frombuffer(pts, np.uint8))
    want = ctx.scalar_mul(curve, sc, pts, HS_AFF, HS_COMPRESSED).reshape(n, 32)
    rec = ctx.scalar_mul(curve, sc, jac, HS_JAC51, HS_JAC51)
    assert (ctx.compress(curve, rec, HS_JAC51).reshape(n, 32) == want).all()
    lib = hs.load()
    fn = lib.hs_helios_scalarmult_vartime if curve == 0 else lib.hs_selene_scalarmult_vartime
    out = np.zeros(120, np.uint8)
    j = np.ascontiguousarray(jac.reshape(n, 120)[3])
    s = np.ascontiguousarray(sc[3])
    fn(out.ctypes.data_as(ctypes.c_void_p), s.ctypes.data_as(ctypes.c_void_p), j.ctypes.data_as(ctypes.c_void_p))
    assert ctx.compress(curve, out, HS_JAC51).tobytes() == want[3].tobytes()
    cls = hs.HeliosPoint if curve == 0 else hs.SelenePoint
    P = cls(j.tobytes())
    assert P.scalar_mul_vartime(bytes(s), ctx).to_bytes(ctx) == want[3].tobytes()
