"""GPU parity: the CUDA MSM path (through the C ABI) against the oracle.

Integer work, so every comparison is bit-exact on the 32-byte serialization
(helios/src/x64/helios_tobytes.cpp:42-66).  The oracle runs in exact mode
(carry kept); where the reference itself is defective (w = 8 band) the GPU
matches the exact sum, which the oracle tests pin to the reference's own
code called on sub-864 chunks.
"""

import ctypes
import random

import numpy as np
import pytest

import oracle
import pyref
from conftest import CURVES, oracle_inputs

pytestmark = pytest.mark.gpu

HS_COMPRESSED, HS_JAC51, HS_AFF51, HS_AFF = 3, 0, 1, 2


def hx(s):
    return bytes.fromhex(s)


def jac51_to_bytes(curve, rec: bytes) -> bytes:
    """encode a 120-byte helios_jacobian record with the oracle"""
    import helioselene_gb300 as hs
    F = pyref.CURVES["helios" if curve == 0 else "selene"].F
    limbs = np.frombuffer(rec, dtype=np.uint64)
    X, Y, Z = (hs.fe51_to_int(limbs[5 * k:5 * k + 5]) % F for k in range(3))
    j96 = X.to_bytes(32, "little") + Y.to_bytes(32, "little") + Z.to_bytes(32, "little")
    return oracle.compress_jac(curve, j96).tobytes()


@pytest.mark.parametrize("curve", [0, 1])
def test_golden_vectors_on_gpu(ctx, golden, curve):
    name = "helios" if curve == 0 else "selene"
    for v in golden[name + "_point"]["msm"]:
        sc = b"".join(hx(s) for s in v["scalars"])
        pts, bad = oracle.decompress(curve, b"".join(hx(s) for s in v["points"]))
        assert ctx.msm(curve, sc, pts, HS_AFF, HS_COMPRESSED).hex() == v["result"], v["label"]
    for v in golden[name + "_point"]["pedersen_commit"]:
        H, _ = oracle.decompress(curve, hx(v["H"]))
        gens, _ = oracle.decompress(curve, b"".join(hx(s) for s in v["generators"]))
        vals = b"".join(hx(s) for s in v["values"])
        assert ctx.pedersen(curve, hx(v["blinding"]), H, vals, gens).hex() == v["result"], v["label"]
    for v in golden[name + "_point"]["map_to_curve_single"]:
        assert ctx.map_to_curve(curve, hx(v["u"]), HS_COMPRESSED).tobytes().hex() == v["result"], v["label"]


@pytest.mark.parametrize("curve", [0, 1])
@pytest.mark.parametrize("n", [1, 2, 7, 16, 17, 33, 64, 100, 257, 1000, 1024, 2048, 4096, 9000])
def test_msm_random(ctx, curve, n):
    sc, pts, _ = oracle_inputs(curve, n, seed=n * 31 + curve)
    assert ctx.msm(curve, sc, pts) == oracle.msm(curve, sc, pts)


@pytest.mark.parametrize("curve", [0, 1])
def test_msm_edge_slices(ctx, curve):
    """zero scalars, order-1, one base repeated with one scalar (bucket doubling), top-window-only"""
    n = 4096
    sc, pts, w = oracle_inputs(curve, n, seed=77, edge_fraction=0.08)
    assert len(w.edge["repeated"]) > 10
    assert ctx.msm(curve, sc, pts) == oracle.msm(curve, sc, pts)


@pytest.mark.parametrize("curve", [0, 1])
def test_msm_degenerate(ctx, curve):
    n = 300
    sc, pts, _ = oracle_inputs(curve, n, seed=5)
    # all-zero scalars -> identity
    assert ctx.msm(curve, np.zeros_like(sc), pts) == bytes(32)
    # n == 0 -> identity in every output format
    assert ctx.msm(curve, sc[:0], pts[:0]) == bytes(32)
    jid = np.frombuffer(ctx.msm(curve, sc[:0], pts[:0], HS_AFF, HS_JAC51), np.uint64)
    assert list(jid) == [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0]
    # identity bases mixed in, P and -P pairs, duplicated points with different scalars,
    # unreduced scalars (bit 255 set, 2^256 - 1)
    pts2 = pts.copy()
    pts2[10:20] = 0
    F = pyref.CURVES["helios" if curve == 0 else "selene"].F
    for i in range(30, 40):
        y = int.from_bytes(pts2[i - 10, 32:].tobytes(), "little")
        pts2[i, :32] = pts2[i - 10, :32]
        pts2[i, 32:] = np.frombuffer(((F - y) % F).to_bytes(32, "little"), np.uint8)
        sc[i] = sc[i - 10]
    pts2[50:60] = pts2[60:70]
    sc[100:110] = 0xFF
    sc[110:120, 31] |= 0x80
    assert ctx.msm(curve, sc, pts2) == oracle.msm(curve, sc, pts2)
    # a sum that cancels to the identity: s*P + s*(-P)
    P = pts[:1].copy()
    mP = P.copy()
    y = int.from_bytes(P[0, 32:].tobytes(), "little")
    mP[0, 32:] = np.frombuffer(((F - y) % F).to_bytes(32, "little"), np.uint8)
    two = np.concatenate([sc[:1], sc[:1]])
    assert ctx.msm(curve, two, np.concatenate([P, mP])) == bytes(32)


@pytest.mark.parametrize("curve", [0, 1])
def test_every_window_width(ctx, curve):
    """the recode is compiled per window width: exercise each c against the oracle"""
    n = 700
    sc, pts, _ = oracle_inputs(curve, n, seed=123, edge_fraction=0.05)
    sc[:7] = 0xFF
    want = oracle.msm(curve, sc, pts)
    try:
        for c in range(4, 21):
            ctx.set_window(curve, 1, 1 << 30, c)
            assert ctx.msm(curve, sc, pts) == want, f"c={c}"
            ctx.set_window(curve, 0, 0, 0)
    finally:
        ctx.set_window(curve, 0, 0, 0)


@pytest.mark.parametrize("curve", [0, 1])
def test_reference_struct_inputs_and_outputs(ctx, curve):
    """helios_jacobian inputs with Z != 1, Z == 0 and lazy limbs; Jacobian output"""
    import helioselene_gb300 as hs
    n = 500
    sc, pts, _ = oracle_inputs(curve, n, seed=8)
    F = pyref.CURVES["helios" if curve == 0 else "selene"].F
    rng = random.Random(4)
    recs, j96 = [], []
    for i in range(n):
        x = int.from_bytes(pts[i, :32].tobytes(), "little")
        y = int.from_bytes(pts[i, 32:].tobytes(), "little")
        if i % 11 == 4:
            X, Y, Z = 1, 1, 0
        elif i % 3 == 0:
            X, Y, Z = x, y, 1
        else:
            z = rng.randrange(2, F)
            X, Y, Z = x * z * z % F, y * z * z * z % F, z
        limbs = hs.int_to_fe51(X) + hs.int_to_fe51(Y) + hs.int_to_fe51(Z)
        if i % 5 == 1 and limbs[1] > 0:
            limbs[1] -= 1
            limbs[0] += 1 << 51
        recs.append(limbs)
        j96.append(X.to_bytes(32, "little") + Y.to_bytes(32, "little") + Z.to_bytes(32, "little"))
    arr = np.array(recs, dtype=np.uint64).view(np.uint8)
    want = oracle.msm_jac(curve, sc, b"".join(j96))
    assert ctx.msm(curve, sc, arr, HS_JAC51, HS_COMPRESSED) == want
    out = ctx.msm(curve, sc, arr, HS_JAC51, HS_JAC51)
    assert jac51_to_bytes(curve, out) == want
    aff = ctx.msm(curve, sc, arr, HS_JAC51, HS_AFF)
    assert oracle.compress(curve, aff).tobytes() == want
    # batch to affine, both output layouts
    got = ctx.batch_to_affine(curve, arr, HS_AFF)
    assert (got == oracle.batch_to_affine(curve, b"".join(j96))).all()
    got51 = ctx.batch_to_affine(curve, arr, HS_AFF51).view(np.uint64).reshape(n, 10)
    for i in range(0, n, 37):
        x = hs.fe51_to_int(got51[i, :5])
        y = hs.fe51_to_int(got51[i, 5:])
        assert x.to_bytes(32, "little") + y.to_bytes(32, "little") == got[64 * i:64 * i + 64].tobytes()
    # compression of Jacobian records
    comp = ctx.compress(curve, arr, HS_JAC51)
    assert (comp == oracle.compress_jac(curve, b"".join(j96))).all()


@pytest.mark.parametrize("curve", [0, 1])
def test_pedersen_random(ctx, curve):
    for n in (1, 16, 1000, 5000):
        sc, pts, _ = oracle_inputs(curve, n + 1, seed=n)
        want = oracle.pedersen(curve, sc[0], pts[0], sc[1:], pts[1:])
        assert ctx.pedersen(curve, sc[0], pts[0], sc[1:], pts[1:]) == want


@pytest.mark.parametrize("curve", [0, 1])
def test_map_to_curve_matches_oracle(ctx, curve):
    from helioselene_gb300.workload import random_field_bytes
    u = random_field_bytes(np.random.default_rng(curve + 40), 2048)
    u[0] = 0
    u[1] = 0xFF  # bit 255 masked by the map
    got = ctx.map_to_curve(curve, u, HS_AFF)
    assert (got == oracle.map_to_curve(curve, u.reshape(-1))).all()


@pytest.mark.parametrize("curve", [0, 1])
def test_reference_signature_dropins(ctx, curve):
    """hs_{helios,selene}_msm_vartime with the reference's argument list"""
    import helioselene_gb300 as hs
    lib = hs.load()
    n = 64
    sc, pts, _ = oracle_inputs(curve, n, seed=64)
    recs = hs.affine64_to_jac51(pts)
    res = np.zeros(15, np.uint64)
    fn = lib.hs_helios_msm_vartime if curve == 0 else lib.hs_selene_msm_vartime
    fn(res.ctypes.data, sc.ctypes.data, recs.ctypes.data, n)
    assert jac51_to_bytes(curve, res.tobytes()) == oracle.msm(curve, sc, pts)
    # n == 0: identity (1:1:0)
    fn(res.ctypes.data, sc.ctypes.data, recs.ctypes.data, 0)
    assert list(res) == [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0]
    # Pedersen drop-in
    ped = lib.hs_helios_pedersen_commit if curve == 0 else lib.hs_selene_pedersen_commit
    ped(res.ctypes.data, sc[0].ctypes.data, recs[:120].ctypes.data, np.ascontiguousarray(sc[1:]).ctypes.data,
        np.ascontiguousarray(recs[120:]).ctypes.data, n - 1)
    assert jac51_to_bytes(curve, res.tobytes()) == oracle.pedersen(curve, sc[0], pts[0], sc[1:], pts[1:])


@pytest.mark.parametrize("curve", [0, 1])
def test_point_api_mirror(ctx, curve):
    import helioselene_gb300 as hs
    Pt = hs.HeliosPoint if curve == 0 else hs.SelenePoint
    n = 40
    sc, pts, _ = oracle_inputs(curve, n, seed=9)
    points = [Pt.from_affine_bytes(pts[i]) for i in range(n)]
    scalars = [sc[i].tobytes() for i in range(n)]
    r = Pt.multi_scalar_mul(scalars, points, ctx)
    assert r.to_bytes(ctx) == oracle.msm(curve, sc, pts)
    assert Pt.multi_scalar_mul([], [], ctx).to_bytes(ctx) == bytes(32)
    c = Pt.pedersen_commit(scalars[0], points[0], scalars[1:], points[1:], ctx)
    assert c.to_bytes(ctx) == oracle.pedersen(curve, sc[0], pts[0], sc[1:], pts[1:])
    aff = (hs.helios_batch_to_affine if curve == 0 else hs.selene_batch_to_affine)(points[:5], ctx)
    assert b"".join(aff) == pts[:5].tobytes()


@pytest.mark.parametrize("curve", [0, 1])
def test_msm_large_vs_threaded_oracle(ctx, curve):
    """n = 2^18 with edge slices, against the oracle run on all host cores"""
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import make_workload
    n = 1 << 18
    w = make_workload(curve, n, seed=2024 + curve, edge_fraction=0.01)
    pts = ctx.map_to_curve(curve, w.u, HS_AFF)
    # the GPU SWU map is itself checked against the oracle on a sample
    idx = np.arange(0, n, 997)
    assert (pts.reshape(n, 64)[idx] == oracle.map_to_curve(curve, w.u[idx].reshape(-1)).reshape(-1, 64)).all()
    got = ctx.msm(curve, w.scalars, pts)
    assert got == oracle.msm_mt(curve, w.scalars, pts, oracle.default_threads())


@pytest.mark.parametrize("curve", [0, 1])
@pytest.mark.parametrize("lg", [20, 22])
def test_linearity_at_full_size(ctx, curve, lg):
    """size-independent property at n = 2^20 and 2^22 (the largest size of the
    sweep): MSM(a) + MSM(b) == MSM(a + b mod order)"""
    from helioselene_gb300.workload import ORDER, make_workload, random_scalars
    n = 1 << lg
    w = make_workload(curve, n, seed=31337 + curve, edge_fraction=0.01)
    pts = ctx.map_to_curve(curve, w.u, HS_AFF)
    a = w.scalars
    b = random_scalars(np.random.default_rng(5), n, ORDER[curve])
    order = ORDER[curve]
    ai = a.view(np.uint64).reshape(n, 4)
    bi = b.view(np.uint64).reshape(n, 4)
    s = np.zeros((n, 4), np.uint64)
    carry = np.zeros(n, np.uint64)
    for i in range(4):
        t = ai[:, i] + bi[:, i]
        c1 = (t < ai[:, i]).astype(np.uint64)
        t2 = t + carry
        c2 = (t2 < t).astype(np.uint64)
        s[:, i] = t2
        carry = c1 | c2
    from helioselene_gb300.workload import below
    over = ~below(s, order)
    o = np.array([(order >> (64 * i)) & (2**64 - 1) for i in range(4)], dtype=np.uint64)
    borrow = np.zeros(n, np.uint64)
    for i in range(4):
        t = s[over, i] - o[i]
        b1 = (s[over, i] < o[i]).astype(np.uint64)
        t2 = t - borrow[over]
        b2 = (t < borrow[over]).astype(np.uint64)
        s[over, i] = t2
        borrow[over] = b1 | b2
    ra = ctx.msm(curve, a, pts, HS_AFF, HS_AFF)
    rb = ctx.msm(curve, b, pts, HS_AFF, HS_AFF)
    rs = ctx.msm(curve, s.view(np.uint8).reshape(n, 32), pts, HS_AFF, HS_COMPRESSED)
    one = np.zeros((2, 32), np.uint8)
    one[:, 0] = 1
    pair = np.frombuffer(ra + rb, np.uint8)
    assert ctx.msm(curve, one, pair) == rs
    assert oracle.compress(curve, oracle.point_add(curve, ra, rb)).tobytes() == rs


@pytest.mark.parametrize("curve", [0, 1])
def test_window_split_matches_unsplit(ctx, curve):
    """single MSMs of n >= 2^18 run as two window halves on two streams joined by
    one addition; the batch path runs the same MSM unsplit.  Odd and even window
    counts, empty upper halves (small scalars) and all-zero scalars."""
    from helioselene_gb300.workload import make_workload
    n = (1 << 18) + 3
    w = make_workload(curve, n, seed=77 + curve, edge_fraction=0.01)
    pts = ctx.map_to_curve(curve, w.u, HS_AFF)
    small = w.scalars.copy()
    small[:, 8:] = 0
    zero = np.zeros_like(w.scalars)
    try:
        for c in (10, 13, 16, 17):
            ctx.set_window(curve, 1, 1 << 30, c)
            for sc in (w.scalars, small, zero):
                split = ctx.msm(curve, sc, pts)
                assert split == ctx.msm_batch([(curve, sc, pts)])[0], f"c={c}"
            ctx.set_window(curve, 0, 0, 0)
    finally:
        ctx.set_window(curve, 0, 0, 0)
    assert ctx.msm(curve, zero, pts) == bytes(32)


def _to_fe51_rows(v32: np.ndarray) -> np.ndarray:
    """(n, 32) little-endian field elements -> (n, 5) radix-2^51 limbs"""
    w = np.ascontiguousarray(v32).view(np.uint64).reshape(-1, 4)
    m = np.uint64((1 << 51) - 1)
    out = np.empty((w.shape[0], 5), np.uint64)
    out[:, 0] = w[:, 0] & m
    out[:, 1] = ((w[:, 0] >> np.uint64(51)) | (w[:, 1] << np.uint64(13))) & m
    out[:, 2] = ((w[:, 1] >> np.uint64(38)) | (w[:, 2] << np.uint64(26))) & m
    out[:, 3] = ((w[:, 2] >> np.uint64(25)) | (w[:, 3] << np.uint64(39))) & m
    out[:, 4] = w[:, 3] >> np.uint64(12)
    return out


@pytest.mark.parametrize("curve", [0, 1])
def test_host_inputs_every_format(ctx, curve):
    """hs_msm / hs_pedersen with host buffers at n = 3 * 2^17 + 1: the inputs
    come over the device's shared copy stream, the scalars first (the sort
    starts on them), the bases converted on a third stream.  Every input
    format, window split on and off, and a Pedersen lead term, against the
    batched path (which stages its inputs whole)."""
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import make_workload
    n = 3 * (1 << 17) + 1
    w = make_workload(curve, n, seed=4242 + curve, edge_fraction=0.01)
    pts = ctx.map_to_curve(curve, w.u, HS_AFF).reshape(n, 64)
    sc = w.scalars
    want = ctx.msm_batch([(curve, sc, pts)])[0]
    # reference records: Z = 1 for most points, random Z for a sample, Z = 0
    # (the identity) for a few, across every part
    F = pyref.CURVES["helios" if curve == 0 else "selene"].F
    x51, y51 = _to_fe51_rows(pts[:, :32]), _to_fe51_rows(pts[:, 32:])
    jac = np.zeros((n, 15), np.uint64)
    jac[:, 0:5], jac[:, 5:10], jac[:, 10] = x51, y51, 1
    rng = random.Random(9)
    for i in range(0, n, 977):
        x = int.from_bytes(pts[i, :32].tobytes(), "little")
        y = int.from_bytes(pts[i, 32:].tobytes(), "little")
        z = rng.randrange(2, F)
        jac[i] = hs.int_to_fe51(x * z * z % F) + hs.int_to_fe51(y * z * z * z % F) + hs.int_to_fe51(z)
    ident = np.arange(5, n, 65537)
    jac[ident] = 0
    jac[ident, 0] = jac[ident, 5] = 1
    pts_id = pts.copy()
    pts_id[ident] = 0
    want_id = ctx.msm_batch([(curve, sc, pts_id)])[0]
    aff51 = np.concatenate([x51, y51], axis=1)
    try:
        # bases in two parts, with XYZZ accumulation or batch-affine rounds (each
        # part's entries of a bucket then in their own padded list)
        for rounds in (0, 1, 2):
            ctx.set_batch_affine(rounds, 1 << 21)
            for split in (1 << 18, 0):
                ctx.set_split(split)
                tag = f"split {split}, rounds {rounds}"
                assert ctx.msm(curve, sc, pts) == want, f"affine, {tag}"
                assert ctx.msm(curve, sc, aff51.view(np.uint8), HS_AFF51) == want, f"affine51, {tag}"
                assert ctx.msm(curve, sc, jac.view(np.uint8), HS_JAC51) == want_id, f"jacobian51, {tag}"
                assert ctx.pedersen(curve, sc[0], pts[0], sc[1:], pts[1:]) == want, f"pedersen, {tag}"
                assert ctx.pedersen(curve, sc[0], jac[0].view(np.uint8), sc[1:], jac[1:].view(np.uint8),
                                    HS_JAC51) == want_id, f"pedersen jacobian51, {tag}"
    finally:
        ctx.set_split(1 << 18)
        ctx.default_batch_affine()


@pytest.mark.parametrize("curve", [0, 1])
def test_host_parts_edge_cases(ctx, curve):
    """host bases in two parts, with the work lopsided between them: every scalar
    of one part zero, a base repeated across both parts with one scalar (one
    bucket of thousands of entries, cut into many segments in each part), and
    identity bases gathered in one part; against the batched path"""
    from helioselene_gb300.workload import make_workload
    n = (1 << 18) + 5
    w = make_workload(curve, n, seed=909 + curve, edge_fraction=0.0)
    pts = ctx.map_to_curve(curve, w.u, HS_AFF).reshape(n, 64).copy()
    half = n // 2
    cases = []
    sc = w.scalars.copy()
    sc[half:] = 0
    cases.append(("second part zero", sc, pts))
    sc = w.scalars.copy()
    sc[:half] = 0
    cases.append(("first part zero", sc, pts))
    sc = w.scalars.copy()
    p2 = pts.copy()
    rep = np.arange(1000, n, 37)
    p2[rep] = pts[1000]
    sc[rep] = sc[1000]
    cases.append(("repeated base across parts", sc, p2))
    p3 = pts.copy()
    p3[: half // 2] = 0
    cases.append(("identity bases in part 0", w.scalars, p3))
    try:
        for rounds in (0, 1, 3):
            ctx.set_batch_affine(rounds, 1 << 20)
            for split in (1 << 18, 0):
                ctx.set_split(split)
                for name, s, p in cases:
                    assert ctx.msm(curve, s, p) == ctx.msm_batch([(curve, s, p)])[0], \
                        f"{name}, split {split}, rounds {rounds}"
    finally:
        ctx.set_split(1 << 18)
        ctx.default_batch_affine()


@pytest.mark.parametrize("curve", [0, 1])
@pytest.mark.parametrize("n", [300, 2000])
def test_small_plan_heavy_buckets(ctx, curve, n):
    """small plans run the eight-lane group kernels (accumulation, merges, window
    reduction): one base repeated with one scalar fills one bucket per window
    with hundreds of entries (many segments: group merges and the heavy-bucket
    path), P and -P with equal scalars cancel inside buckets, and equal points
    with equal scalars double in the mixed addition"""
    sc, pts, _ = oracle_inputs(curve, n, seed=400 + n + curve)
    F = pyref.CURVES["helios" if curve == 0 else "selene"].F
    rep = n // 3
    pts[1:rep] = pts[0]
    sc[1:rep] = sc[0]
    for i in range(rep, rep + 40, 2):  # P, -P pairs with one scalar
        y = int.from_bytes(pts[i, 32:].tobytes(), "little")
        pts[i + 1, :32] = pts[i, :32]
        pts[i + 1, 32:] = np.frombuffer(((F - y) % F).to_bytes(32, "little"), np.uint8)
        sc[i + 1] = sc[i]
    assert ctx.msm(curve, sc, pts) == oracle.msm(curve, sc, pts)
    assert ctx.msm_batch([(curve, sc, pts), (curve, sc[: n // 2], pts[: n // 2])]) == [
        oracle.msm(curve, sc, pts), oracle.msm(curve, sc[: n // 2], pts[: n // 2])]


def _placed(data: np.ndarray, offset: int, pinned: bool = False) -> np.ndarray:
    """a copy of the bytes of `data` starting `offset` bytes past a 16-byte
    boundary, in pageable (numpy) or pinned (torch) host memory"""
    raw = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    if pinned:
        import torch
        buf = torch.empty(raw.size + 32, dtype=torch.uint8, pin_memory=True).numpy()
    else:
        buf = np.empty(raw.size + 32, np.uint8)
    base = (-buf.ctypes.data) % 16
    view = buf[base + offset:base + offset + raw.size]
    view[:] = raw
    return view


@pytest.mark.parametrize("curve", [0, 1])
def test_host_buffers_pinned_pageable_unaligned(ctx, curve):
    """Host inputs in pageable memory -- pulled by a copy kernel that reads the
    caller's pages where the device reads pageable memory, by the copy engine
    elsewhere -- at byte offsets 0, 1, 4 and 8 from a 16-byte boundary (the
    kernel's 16-, 8-, 4- and 1-byte word forms, with ragged tails), and in
    pinned memory (copy engine): single MSMs with the bases in two parts,
    Pedersen with its lead term, and host batches of 3 and of 20 MSMs (the
    latter a gathered copy kernel from either memory), against the oracle."""
    n = (1 << 18) + 3
    from helioselene_gb300.workload import make_workload
    w = make_workload(curve, n, seed=5150 + curve, edge_fraction=0.01)
    pts = ctx.map_to_curve(curve, w.u, HS_AFF).reshape(n, 64)
    sc = w.scalars.reshape(n, 32)
    want = oracle.msm_mt(curve, sc, pts, oracle.default_threads())
    jac = np.zeros((n, 15), np.uint64)
    jac[:, 0:5], jac[:, 5:10], jac[:, 10] = _to_fe51_rows(pts[:, :32]), _to_fe51_rows(pts[:, 32:]), 1
    sizes = (1000, 77, 2001)
    cuts = np.cumsum((0,) + sizes)
    want_small = [oracle.msm(curve, sc[a:b], pts[a:b]) for a, b in zip(cuts[:-1], cuts[1:])]
    # more than 16 MSMs in a group: one gathered copy kernel whatever the memory
    many = np.cumsum([0] + [37 + 11 * i for i in range(20)])
    want_many = [oracle.msm(curve, sc[a:b], pts[a:b]) for a, b in zip(many[:-1], many[1:])]
    counts = {}
    for pinned, offsets in ((False, (0, 1, 4, 8)), (True, (0, 1))):
        for off in offsets:
            tag = f"{'pinned' if pinned else 'pageable'} offset {off}"
            s_v = _placed(sc, off, pinned)
            j_v = _placed(jac, off, pinned)
            p_v = _placed(pts, off, pinned)
            before = ctx.launches
            assert ctx.msm(curve, s_v, j_v, HS_JAC51) == want, tag
            counts[(pinned, off)] = ctx.launches - before
            assert ctx.msm(curve, s_v, p_v, HS_AFF) == want, tag
            assert ctx.pedersen(curve, s_v[:32], p_v[:64], s_v[32:], p_v[64:]) == want, f"pedersen, {tag}"
            items = [(curve, s_v[32 * a:32 * b], p_v[64 * a:64 * b]) for a, b in zip(cuts[:-1], cuts[1:])]
            assert ctx.msm_batch(items) == want_small, f"batch, {tag}"
            items = [(curve, s_v[32 * a:32 * b], p_v[64 * a:64 * b]) for a, b in zip(many[:-1], many[1:])]
            assert ctx.msm_batch(items) == want_many, f"batch of 20, {tag}"
    # a pageable call launches the same sequence as a pinned one, plus one copy
    # kernel per input copy (scalars and two parts of bases) where the device
    # reads pageable memory
    extra = {counts[(False, off)] - counts[(True, 0)] for off in (0, 1, 4, 8)}
    assert extra in ({0}, {3}), counts
