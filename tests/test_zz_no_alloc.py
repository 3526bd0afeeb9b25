"""hs_msm_device_noalloc: the MSM for callers that cannot allocate device memory
while they run (an allocator that must not be bypassed, memory reserved up
front, or code that must never reach cudaMalloc/cudaFree).  It takes all its
scratch from one fixed device array, so its results are checked against the
allocating entry point hs_msm_device on consecutive calls -- the second call
finds the first call's leftovers in the shared array and must not be affected.
Collected last on purpose (test_zz_*), and self-contained so it also passes
alone in a fresh process."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HS_ERANGE, HS_COMPRESSED, HS_JAC51 = -6, 3, 0


def _inputs(curve, n, seed):
    import oracle
    from helioselene_gb300.workload import make_workload
    w = make_workload(curve, n, seed, edge_fraction=0.02)
    return w.scalars.reshape(-1), oracle.map_to_curve(curve, w.u.reshape(-1))


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    lib = hs.load()
    ctx = hs.Context(0)
    try:
        stream = torch.cuda.current_stream()
        cases = [(hs.HELIOS, 20000, 1), (hs.HELIOS, 3000, 2), (hs.SELENE, 20000, 3), (hs.SELENE, 777, 4)]
        for curve, n, seed in cases:
            sc, pts = _inputs(curve, n, seed)
            d_sc = torch.from_numpy(sc).cuda()
            d_pts = torch.from_numpy(pts).cuda()
            d_a = torch.zeros(32, dtype=torch.uint8, device="cuda")
            d_b = torch.zeros(32, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            rc = lib.hs_msm_device_noalloc(curve, ctypes.c_void_p(d_sc.data_ptr()), ctypes.c_void_p(d_pts.data_ptr()),
                                           n, ctypes.c_void_p(d_a.data_ptr()), HS_COMPRESSED,
                                           ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0
            torch.cuda.synchronize()
            ctx.msm_device(curve, d_sc.data_ptr(), d_pts.data_ptr(), n, d_b.data_ptr(), HS_COMPRESSED)
            torch.cuda.ExternalStream(ctx.stream).synchronize()
            assert d_a.cpu().numpy().tobytes() == d_b.cpu().numpy().tobytes(), (curve, n)
    finally:
        ctx.close()


def test_noalloc_limits():
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    lib = hs.load()
    assert lib.hs_msm_noalloc_scratch_bytes() == 64 << 20
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    too_many = 262144 + 1
    rc = lib.hs_msm_device_noalloc(0, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()), too_many,
                                   ctypes.c_void_p(d.data_ptr()), HS_COMPRESSED, None)
    assert rc == HS_ERANGE
    rc = lib.hs_msm_device_noalloc(0, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()), 0,
                                   ctypes.c_void_p(d.data_ptr()), HS_COMPRESSED, None)
    assert rc == HS_ERANGE


def test_noalloc_at_the_size_limit():
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import make_workload
    lib = hs.load()
    ctx = hs.Context(0)
    try:
        n = 262144
        w = make_workload(hs.SELENE, n, 99, edge_fraction=0.01)
        d_u = torch.from_numpy(w.u.reshape(-1).copy()).cuda()
        d_pts = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
        d_sc = torch.from_numpy(w.scalars.reshape(-1).copy()).cuda()
        torch.cuda.synchronize()
        ctx.map_to_curve_device(hs.SELENE, d_u.data_ptr(), n, d_pts.data_ptr())
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        d_a = torch.zeros(120, dtype=torch.uint8, device="cuda")
        d_b = torch.zeros(120, dtype=torch.uint8, device="cuda")
        for _ in range(2):
            rc = lib.hs_msm_device_noalloc(hs.SELENE, ctypes.c_void_p(d_sc.data_ptr()),
                                           ctypes.c_void_p(d_pts.data_ptr()), n, ctypes.c_void_p(d_a.data_ptr()),
                                           HS_JAC51, None)
            assert rc == 0
            torch.cuda.synchronize()
            ctx.msm_device(hs.SELENE, d_sc.data_ptr(), d_pts.data_ptr(), n, d_b.data_ptr(), HS_JAC51)
            torch.cuda.ExternalStream(ctx.stream).synchronize()
            a = ctx.compress(hs.SELENE, d_a.cpu().numpy(), HS_JAC51)
            b = ctx.compress(hs.SELENE, d_b.cpu().numpy(), HS_JAC51)
            assert (a == b).all()
    finally:
        ctx.close()
