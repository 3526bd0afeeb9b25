"""GPU parity at the sizes of every benchmark configuration, against the oracle.

Each test builds the benchmark's own seeded inputs (helioselene_gb300.workload)
and compares every result bit for bit on the 32-byte serialization:

* single MSMs n = 2^10, 2^12, ..., 2^22 on both curves with the 1% edge slices
  (zero scalars, order-1, one base repeated with one scalar, top-window-only),
  device-resident inputs through hs_msm_device with the library's defaults;
* the batched stream: 1024 MSMs of log-uniform sizes in [64, 65536] on either
  curve, one hs_msm_batch_device call per curve, every MSM checked;
* the serving mixture (70% [256, 4096], 25% [4096, 65536], 5% 2^18 points)
  over a 2^18-point resident pool per curve plus fresh bases, a seeded subset
  of requests submitted at once to a continuous-batching server;
* fixed-base commitments over 2^20 generators and H: dense and sparse
  (<= 16 set bits) scalars, affine outputs.

The oracle's multi-threaded forms (per-thread sub-MSMs summed with the group
law, or one MSM per thread) keep the large sizes within seconds.  The SWU map
that makes the bases runs on the GPU and is itself checked on a sample.
"""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HS_COMPRESSED, HS_JAC51, HS_AFF = 3, 0, 2


def _device_bases(torch, ctx, curve, u):
    """SWU images of u computed on the device (d_pts), checked against the oracle on a sample"""
    n = u.shape[0]
    d_u = torch.from_numpy(np.ascontiguousarray(u).reshape(-1)).cuda()
    d_pts = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.map_to_curve_device(curve, d_u.data_ptr(), n, d_pts.data_ptr())
    torch.cuda.ExternalStream(ctx.stream).synchronize()
    pts = d_pts.cpu().numpy().reshape(n, 64)
    idx = np.unique(np.concatenate([np.arange(0, n, max(1, n // 64)), [n - 1]]))
    assert (pts[idx] == oracle.map_to_curve(curve, u[idx].reshape(-1)).reshape(-1, 64)).all()
    return d_pts, pts


@pytest.mark.parametrize("curve", [0, 1])
def test_single_msm_sweep_with_edge_slices(ctx, curve):
    torch = pytest.importorskip("torch")
    from helioselene_gb300.workload import BENCH_SEED, make_workload
    threads = oracle.default_threads()
    d_out = torch.empty(128, dtype=torch.uint8, device="cuda")
    for lg in range(10, 23, 2):
        n = 1 << lg
        w = make_workload(curve, n, BENCH_SEED + 2 + lg, edge_fraction=0.01)
        assert len(w.edge["repeated"]) >= 2
        d_pts, pts = _device_bases(torch, ctx, curve, w.u)
        d_sc = torch.from_numpy(w.scalars.reshape(-1).copy()).cuda()
        torch.cuda.synchronize()
        ctx.msm_device(curve, d_sc.data_ptr(), d_pts.data_ptr(), n, d_out.data_ptr(), HS_JAC51)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        got = ctx.compress(curve, d_out[:120].cpu().numpy(), HS_JAC51).tobytes()
        want = oracle.msm_mt(curve, w.scalars, pts, threads)
        assert got == want, f"n=2^{lg}"
        del d_pts, d_sc


def test_batched_stream_of_1024_msms(ctx):
    torch = pytest.importorskip("torch")
    from helioselene_gb300.workload import batched_stream
    bs = batched_stream()
    assert bs["sizes"].size == 1024 and bs["sizes"].min() >= 64 and bs["sizes"].max() <= 65536
    for curve in (0, 1):
        g = bs[curve]
        m = len(g["sizes"])
        d_pts, pts = _device_bases(torch, ctx, curve, g["u"])
        d_sc = torch.from_numpy(g["scalars"].reshape(-1).copy()).cuda()
        d_out = torch.empty(m * 120, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.msm_batch_device(curve, g["sizes"], d_sc.data_ptr(), d_pts.data_ptr(), d_out.data_ptr(), HS_JAC51)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        got = ctx.compress(curve, d_out.cpu().numpy(), HS_JAC51).reshape(m, 32)
        want = oracle.msm_many(curve, g["scalars"], pts, g["sizes"])
        bad = [i for i in range(m) if got[i].tobytes() != want[i]]
        assert not bad, f"curve {curve}: {len(bad)} of {m} MSMs differ, e.g. sizes {[g['sizes'][i] for i in bad[:5]]}"
        del d_pts, d_sc


def test_serving_mixture_over_a_2p18_pool():
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import BENCH_SEED, ORDER, random_field_bytes, random_scalars, serving_sizes
    rng = np.random.default_rng(BENCH_SEED + 40)
    pool_n = 1 << 18
    ctx = hs.Context(0)
    try:
        pools = {}
        for curve in (0, 1):
            _, pools[curve] = _device_bases(torch, ctx, curve, random_field_bytes(rng, pool_n))
    finally:
        ctx.close()
    count = 96
    sizes = serving_sizes(rng, count)
    sizes[:4] = 1 << 18  # the 2^18 requests of the mixture, on both curves, certainly in the subset
    reqs = []
    for i, k in enumerate(sizes):
        curve = i % 2
        k = int(k)
        npool = (3 * k) // 4
        nfresh = k - npool
        idx = rng.integers(0, pool_n, npool).astype(np.uint32)
        fresh = oracle.map_to_curve(curve, random_field_bytes(rng, nfresh).reshape(-1)).reshape(nfresh, 64)
        sc = random_scalars(rng, k, ORDER[curve])
        reqs.append((curve, sc, idx, fresh))
    with hs.Server(0, slots=8, max_batch_points=1 << 23, max_batch_msms=1024) as srv:
        for c in (0, 1):
            srv.set_pool(c, pools[c])
        tickets = [srv.submit(c, sc, idx, fr) for c, sc, idx, fr in reqs]
        got = [srv.wait(t, 600000)[0] for t in tickets]
        st = srv.stats()
    assert st["completed"] == count and st["failed"] == 0
    for curve in (0, 1):
        sel = [i for i in range(count) if reqs[i][0] == curve]
        sc = np.concatenate([reqs[i][1] for i in sel])
        pts = np.concatenate([np.concatenate([pools[curve][reqs[i][2]], reqs[i][3]]) for i in sel])
        want = oracle.msm_many(curve, sc, pts, [int(sizes[i]) for i in sel])
        bad = [sel[j] for j in range(len(sel)) if got[sel[j]] != want[j]]
        assert not bad, f"curve {curve}: requests {bad[:8]} differ (sizes {[int(sizes[i]) for i in bad[:8]]})"


@pytest.mark.parametrize("curve", [0, 1])
def test_fixed_base_commitments_over_2p20_generators(curve):
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import BENCH_SEED, ORDER, random_field_bytes, random_scalars
    n = 1 << 20
    rng = np.random.default_rng(BENCH_SEED + 50 + curve)
    ctx = hs.Context(0)
    try:
        _, gens = _device_bases(torch, ctx, curve, random_field_bytes(rng, n + 1))
        fb = hs.FixedBase(ctx, curve, gens[:n], H=gens[n])
        dense, sparse = 8, 4
        count = dense + sparse
        sc = random_scalars(rng, count * (n + 1), ORDER[curve]).reshape(count, n + 1, 32)
        # sparse scalars: one 16-bit value at a random byte offset (<= 16 set bits)
        sp = sc[dense:]
        sp[:] = 0
        v16 = rng.integers(0, 65536, (sparse, n + 1))
        off = rng.integers(0, 30, (sparse, n + 1))
        r, c = np.meshgrid(np.arange(sparse), np.arange(n + 1), indexing="ij")
        sp[r, c, off] = (v16 & 0xFF).astype(np.uint8)
        sp[r, c, off + 1] = (v16 >> 8).astype(np.uint8)
        d_sc = torch.from_numpy(sc.reshape(-1)).cuda()
        d_out = torch.empty(count * 64, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        fb.commit_device(d_sc.data_ptr(), count, d_out.data_ptr(), HS_AFF)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        got = ctx.compress(curve, d_out.cpu().numpy(), HS_AFF).reshape(count, 32)
        fb.close()
        threads = oracle.default_threads()
        for j in range(count):
            # blinding last in each commitment's scalars, H appended as generator n
            want = oracle.msm_mt(curve, sc[j], gens, threads)
            assert got[j].tobytes() == want, f"commitment {j} ({'sparse' if j >= dense else 'dense'})"
    finally:
        ctx.close()
