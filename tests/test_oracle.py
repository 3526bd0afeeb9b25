"""The oracle against the reference: golden vectors, the Python big-int model and
(where it was compiled here) the reference library itself.  CPU only."""

import ctypes
import random

import numpy as np
import pytest

import oracle
import pyref
from conftest import CURVES, ROOT, oracle_inputs

REF_LIB = ROOT / "oracle" / "_ref" / "libhsref.so"


def hx(s):
    return bytes.fromhex(s)


@pytest.fixture(scope="module")
def ref():
    if not REF_LIB.exists():
        pytest.skip("reference library not compiled here (needs the reference sources)")
    lib = ctypes.CDLL(str(REF_LIB))
    for name in ("ref_msm", "ref_map_to_curve", "ref_pedersen", "ref_batch_to_affine", "ref_msm_jac51",
                 "ref_encode_jac51"):
        getattr(lib, name).restype = ctypes.c_int
    return lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("curve", list(CURVES))
def test_golden_msm(golden, curve):
    for v in golden[curve + "_point"]["msm"]:
        sc = b"".join(hx(s) for s in v["scalars"])
        pts, bad = oracle.decompress(curve, b"".join(hx(s) for s in v["points"]))
        assert bad == 0
        assert oracle.msm(curve, sc, pts, keep_carry=False).hex() == v["result"], v["label"]
        assert oracle.msm(curve, sc, pts, keep_carry=True).hex() == v["result"], v["label"]


@pytest.mark.parametrize("curve", list(CURVES))
def test_golden_pedersen(golden, curve):
    for v in golden[curve + "_point"]["pedersen_commit"]:
        H, _ = oracle.decompress(curve, hx(v["H"]))
        gens, bad = oracle.decompress(curve, b"".join(hx(s) for s in v["generators"]))
        assert bad == 0
        vals = b"".join(hx(s) for s in v["values"])
        assert oracle.pedersen(curve, hx(v["blinding"]), H, vals, gens).hex() == v["result"], v["label"]


@pytest.mark.parametrize("curve", list(CURVES))
def test_golden_map_to_curve(golden, curve):
    for v in golden[curve + "_point"]["map_to_curve_single"]:
        a = oracle.map_to_curve(curve, hx(v["u"]))
        assert oracle.compress(curve, a).tobytes().hex() == v["result"], v["label"]


@pytest.mark.parametrize("curve", list(CURVES))
def test_golden_group_law(golden, curve):
    gp = golden[curve + "_point"]
    for v in gp["scalar_mul"]:
        P, _ = oracle.decompress(curve, hx(v["point"]))
        r = oracle.scalar_mul(curve, hx(v["scalar"]), P)
        assert oracle.compress(curve, r).tobytes().hex() == v["result"], v["label"]
    for v in gp["add"]:
        a, _ = oracle.decompress(curve, hx(v["a"]))
        b, _ = oracle.decompress(curve, hx(v["b"]))
        assert oracle.compress(curve, oracle.point_add(curve, a, b)).tobytes().hex() == v["result"], v["label"]
    for v in gp["from_bytes"]:
        a, bad = oracle.decompress(curve, hx(v["input"]))
        if v["result"] is None or v["result"] == "invalid" or v["result"] == "":
            assert bad == 1, v["label"]
        else:
            assert bad == 0 and oracle.compress(curve, a).tobytes().hex() == v["result"], v["label"]


def test_golden_batch_invert(golden):
    for field, fid in (("fp", oracle.FIELD_P), ("fq", oracle.FIELD_Q)):
        for v in golden["batch_invert"][field]:
            out = oracle.batch_invert(fid, b"".join(hx(s) for s in v["inputs"]))
            assert [out[32 * i:32 * i + 32].tobytes().hex() for i in range(v["n"])] == v["results"], v["label"]


@pytest.mark.parametrize("curve", list(CURVES))
def test_oracle_matches_bigint_model(curve):
    C = pyref.CURVES[curve]
    rng = random.Random(7)
    for n in (1, 3, 17, 40):
        us = [rng.randbytes(32) for _ in range(n)]
        sc = [rng.getrandbits(256) for _ in range(n)]
        pts = oracle.map_to_curve(curve, b"".join(us))
        mpts = [C.map_to_curve(u) for u in us]
        for i in range(n):
            x, y = mpts[i]
            assert pts[64 * i:64 * i + 64].tobytes() == x.to_bytes(32, "little") + y.to_bytes(32, "little")
        scb = b"".join(s.to_bytes(32, "little") for s in sc)
        assert oracle.msm(curve, scb, pts) == C.encode(C.msm(sc, mpts))


@pytest.mark.parametrize("curve", list(CURVES))
@pytest.mark.parametrize("n", [5, 17, 100, 300, 900, 1024, 2048, 2600, 8000])
def test_oracle_matches_reference_library(ref, curve, n):
    cid = CURVES[curve]
    sc, pts, _ = oracle_inputs(cid, n, seed=1000 + n, edge_fraction=0.04 if n >= 100 else 0.0)
    out = np.zeros(32, np.uint8)
    assert ref.ref_msm(cid, _p(out), _p(sc), _p(pts), ctypes.c_size_t(n)) == 0
    r_ref = out.tobytes()
    # keep_carry = 0 is the reference bit for bit, including the w = 8 band
    assert oracle.msm(cid, sc, pts, keep_carry=False) == r_ref
    exact = oracle.msm(cid, sc, pts, keep_carry=True)
    if not 864 <= n < 2592:
        assert exact == r_ref
    # exact mode equals the reference's own MSM called on chunks below the w = 8 band
    # (n < 864), summed with the group law
    if 864 <= n < 2592:
        acc = np.zeros(64, np.uint8)
        for lo in range(0, n, 800):
            hi = min(n, lo + 800)
            o = np.zeros(32, np.uint8)
            ref.ref_msm(cid, _p(o), _p(np.ascontiguousarray(sc[lo:hi])), _p(np.ascontiguousarray(pts[lo:hi])),
                        ctypes.c_size_t(hi - lo))
            part, bad = oracle.decompress(cid, o.tobytes())
            assert bad == 0
            acc = np.frombuffer(oracle.point_add(cid, acc, part), np.uint8)
        assert oracle.compress(cid, acc).tobytes() == exact


@pytest.mark.parametrize("curve", list(CURVES))
def test_reference_w8_defect_is_reproduced(ref, curve):
    """864 <= n < 2592: the reference drops 2^256 * P_i for scalars whose recode carries
    out of digit 31 (helios_msm_vartime.cpp:127-162); exact mode does not."""
    cid = CURVES[curve]
    n = 1024
    sc, pts, _ = oracle_inputs(cid, n, seed=99)
    sc[:, 31] = 0x7F  # top byte 0x7f: digit 31 is >= 128 after any carry, so the carry is dropped
    out = np.zeros(32, np.uint8)
    ref.ref_msm(cid, _p(out), _p(sc), _p(pts), ctypes.c_size_t(n))
    assert oracle.msm(cid, sc, pts, keep_carry=False) == out.tobytes()
    assert oracle.msm(cid, sc, pts, keep_carry=True) != out.tobytes()
    assert oracle.msm(cid, sc, pts, keep_carry=True) == oracle.msm_naive(cid, sc, pts)


@pytest.mark.parametrize("curve", list(CURVES))
def test_reference_pedersen_and_map(ref, curve):
    cid = CURVES[curve]
    sc, pts, w = oracle_inputs(cid, 33, seed=5)
    out = np.zeros(32, np.uint8)
    ref.ref_pedersen(cid, _p(out), _p(sc[0]), _p(pts[0]), _p(np.ascontiguousarray(sc[1:])),
                     _p(np.ascontiguousarray(pts[1:])), ctypes.c_size_t(32))
    assert oracle.pedersen(cid, sc[0], pts[0], sc[1:], pts[1:]) == out.tobytes()
    for i in range(8):
        ref.ref_map_to_curve(cid, _p(out), _p(np.ascontiguousarray(w.u[i])))
        assert oracle.compress(cid, pts[i]).tobytes() == out.tobytes()


@pytest.mark.parametrize("curve", list(CURVES))
def test_reference_jacobian51_inputs(ref, curve):
    """Z != 1, identity (Z = 0) and lazy limbs in the reference's own struct."""
    import helioselene_gb300 as hs
    cid = CURVES[curve]
    C = pyref.CURVES[curve]
    F = C.F
    n = 40
    sc, pts, _ = oracle_inputs(cid, n, seed=11)
    rng = random.Random(3)
    recs, jac96 = [], []
    for i in range(n):
        x = int.from_bytes(pts[i, :32].tobytes(), "little")
        y = int.from_bytes(pts[i, 32:].tobytes(), "little")
        if i % 7 == 3:
            X, Y, Z = 1, 1, 0
        else:
            z = rng.randrange(1, F)
            X, Y, Z = x * z * z % F, y * z * z * z % F, z
        limbs = hs.int_to_fe51(X) + hs.int_to_fe51(Y) + hs.int_to_fe51(Z)
        if i % 5 == 1:  # lazy (non-canonical) limb: borrow 2^51 from limb 1 into limb 0
            if limbs[1] > 0:
                limbs[1] -= 1
                limbs[0] += 1 << 51
        recs.append(limbs)
        jac96.append(X.to_bytes(32, "little") + Y.to_bytes(32, "little") + Z.to_bytes(32, "little"))
    arr = np.array(recs, dtype=np.uint64)
    out = np.zeros(32, np.uint8)
    assert ref.ref_msm_jac51(cid, _p(out), _p(sc), _p(arr), ctypes.c_size_t(n)) == 0
    assert oracle.msm_jac(cid, sc, b"".join(jac96)) == out.tobytes()
    # batch to affine
    aff = np.zeros(64 * n, np.uint8)
    ref.ref_batch_to_affine(cid, _p(aff), _p(arr), ctypes.c_size_t(n))
    assert (oracle.batch_to_affine(cid, b"".join(jac96)) == aff).all()


def test_fe51_conversion():
    import helioselene_gb300 as hs
    for field, m in ((oracle.FIELD_P, pyref.P), (oracle.FIELD_Q, pyref.Q)):
        for v in (0, 1, m - 1, m, m + 5, 2**255 - 1, 2**256 - 1):
            limbs = hs.int_to_fe51(v % 2**255) if v < 2**255 else [2**51 - 1] * 4 + [2**53 - 1]
            val = hs.fe51_to_int(limbs)
            assert oracle.fe51_to_bytes(field, limbs) == (val % m).to_bytes(32, "little")


@pytest.mark.parametrize("curve", list(CURVES))
def test_unreduced_and_degenerate_scalars(curve):
    cid = CURVES[curve]
    n = 20
    sc, pts, _ = oracle_inputs(cid, n, seed=21)
    sc[:5] = 0xFF  # 2^256 - 1: any 32-byte value is accepted
    sc[5:8] = 0
    exact = oracle.msm(cid, sc, pts)
    assert exact == oracle.msm_naive(cid, sc, pts)
    assert oracle.msm(cid, np.zeros_like(sc), pts) == bytes(32)
    assert oracle.msm(cid, sc[:0], pts[:0]) == bytes(32)
