"""Batched MSMs (one launch sequence for many uneven MSMs, either curve) against
the oracle, MSM by MSM; graph replay with fresh data; per-size window rules."""

import ctypes

import numpy as np
import pytest

import oracle
from conftest import oracle_inputs

pytestmark = pytest.mark.gpu

HS_JAC51, HS_AFF, HS_COMPRESSED = 0, 2, 3


def _batch(seed, sizes, curves, edge=0.0):
    items, want = [], []
    for i, (n, c) in enumerate(zip(sizes, curves)):
        sc, pts, _ = oracle_inputs(c, n, seed=seed + i, edge_fraction=edge) if n else (
            np.zeros((0, 32), np.uint8), np.zeros((0, 64), np.uint8), None)
        items.append((c, sc, pts))
        want.append(oracle.msm(c, sc, pts) if n else bytes(32))
    return items, want


def test_host_batch_mixed_curves(ctx):
    rng = np.random.default_rng(3)
    sizes = [0, 1, 2, 16, 17, 64, 100, 333, 1000, 4096, 20000] + list(
        np.exp(rng.uniform(np.log(64), np.log(8192), 30)).astype(int))
    curves = list(rng.integers(0, 2, len(sizes)))
    items, want = _batch(500, sizes, curves, edge=0.04)
    got = ctx.msm_batch(items, HS_AFF, HS_COMPRESSED)
    bad = [i for i, (g, w) in enumerate(zip(got, want)) if g != w]
    assert not bad, f"mismatching MSMs: {bad[:10]}"


@pytest.mark.parametrize("batch", [1, 4, 10])
def test_fcmpp_verification_shapes(ctx, batch):
    """FCMP++ verification of `batch` proofs (src/benchmark_fcmpp.cpp:350-439):
    one Selene MSM of 522 + 80*batch terms and one Helios MSM of 265 + 80*batch,
    as two single calls from reference records and as one mixed-curve batch of
    three verifications; batch = 10 puts both sizes in the reference's w = 8
    band, where the GPU gives the exact sum."""
    import helioselene_gb300 as hs
    sizes = [522 + 80 * batch, 265 + 80 * batch] * 3
    items, want = _batch(4000 + batch, sizes, [1, 0] * 3)
    for (c, sc, pts), w in list(zip(items, want))[:2]:
        assert ctx.msm(c, sc, hs.affine64_to_jac51(pts), HS_JAC51, HS_COMPRESSED) == w
    assert ctx.msm_batch(items, HS_AFF, HS_COMPRESSED) == want


def test_host_batch_reference_records(ctx):
    import helioselene_gb300 as hs
    sizes = [5, 300, 2000]
    items, want = _batch(900, sizes, [0, 1, 0])
    items51 = [(c, sc, hs.affine64_to_jac51(pts)) for c, sc, pts in items]
    got = ctx.msm_batch(items51, HS_JAC51, HS_COMPRESSED)
    assert got == want


@pytest.mark.parametrize("curve", [0, 1])
def test_device_batch_and_graph_replay(ctx, curve):
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    rng = np.random.default_rng(11 + curve)
    sizes = [int(x) for x in np.exp(rng.uniform(np.log(64), np.log(20000), 24)).astype(int)]
    total = sum(sizes)
    for rep in range(3):
        items, want = _batch(1000 * rep + 77 * curve, sizes, [curve] * len(sizes))
        sc = np.concatenate([s for _, s, _ in items]).reshape(-1)
        pts = np.concatenate([p for _, _, p in items]).reshape(-1)
        d_sc = torch.from_numpy(sc).cuda()
        d_pts = torch.from_numpy(pts).cuda()
        d_out = torch.zeros(32 * len(sizes), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.msm_batch_device(curve, sizes, d_sc.data_ptr(), d_pts.data_ptr(), d_out.data_ptr(), HS_COMPRESSED)
        stream = torch.cuda.ExternalStream(ctx.stream)
        stream.synchronize()
        out = d_out.cpu().numpy().reshape(-1, 32)
        got = [out[i].tobytes() for i in range(len(sizes))]
        assert got == want, f"rep {rep}"
        assert total == d_sc.numel() // 32


def test_per_size_window_rules_in_one_batch(ctx):
    sizes = [100, 700, 3000, 9000]
    items, want = _batch(4242, sizes, [1] * 4, edge=0.05)
    try:
        ctx.set_window(1, 1, 500, 5)
        ctx.set_window(1, 501, 2000, 13)
        ctx.set_window(1, 2001, 5000, 8)
        ctx.set_window(1, 5001, 1 << 30, 17)
        assert ctx.msm_batch(items, HS_AFF, HS_COMPRESSED) == want
    finally:
        ctx.set_window(1, 0, 0, 0)
