"""hs_msm_device_noalloc: the MSM for callers that cannot allocate device memory
while they run (an allocator that must not be bypassed, memory reserved up
front, or code that must never reach cudaMalloc/cudaFree).  It takes all its
scratch from one fixed device array, so its results are checked against the
allocating entry point hs_msm_device and against the oracle on consecutive
calls -- the second call finds the first call's leftovers in the shared array
and must not be affected -- and the free device memory is checked to stay
the same across calls.  Collected last on purpose (test_zz_*), and
self-contained so it also passes alone in a fresh process."""

import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HS_ERANGE, HS_COMPRESSED, HS_JAC51 = -6, 3, 0
MAX_POINTS = 262144


def _inputs(curve, n, seed):
    from helioselene_gb300.workload import make_workload
    w = make_workload(curve, n, seed, edge_fraction=0.02)
    return w.scalars.reshape(-1), oracle.map_to_curve(curve, w.u.reshape(-1))


def _noalloc(lib, curve, d_sc, d_pts, n, d_out, fmt, stream):
    return lib.hs_msm_device_noalloc(curve, ctypes.c_void_p(d_sc.data_ptr()), ctypes.c_void_p(d_pts.data_ptr()), n,
                                     ctypes.c_void_p(d_out.data_ptr()), fmt, stream)


def test_noalloc_matches_allocating_entry_point_and_oracle_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    lib = hs.load()
    ctx = hs.Context(0)
    try:
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        cases = [(hs.HELIOS, 20000, 1), (hs.HELIOS, 3000, 2), (hs.SELENE, 20000, 3), (hs.SELENE, 777, 4)]
        for curve, n, seed in cases:
            sc, pts = _inputs(curve, n, seed)
            want = oracle.msm(curve, sc, pts)
            d_sc = torch.from_numpy(sc).cuda()
            d_pts = torch.from_numpy(pts).cuda()
            d_b = torch.zeros(32, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            ctx.msm_device(curve, d_sc.data_ptr(), d_pts.data_ptr(), n, d_b.data_ptr(), HS_COMPRESSED)
            torch.cuda.ExternalStream(ctx.stream).synchronize()
            for _ in range(2):
                d_a = torch.zeros(32, dtype=torch.uint8, device="cuda")
                torch.cuda.synchronize()
                assert _noalloc(lib, curve, d_sc, d_pts, n, d_a, HS_COMPRESSED, stream) == 0
                torch.cuda.synchronize()
                got = d_a.cpu().numpy().tobytes()
                assert got == d_b.cpu().numpy().tobytes(), (curve, n)
                assert got == want, (curve, n)
    finally:
        ctx.close()


def test_noalloc_limits():
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    lib = hs.load()
    assert lib.hs_msm_noalloc_scratch_bytes() == 64 << 20
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    for curve in (hs.HELIOS, hs.SELENE):
        for n in (MAX_POINTS + 1, 0):
            assert _noalloc(lib, curve, d, d, n, d, HS_COMPRESSED, None) == HS_ERANGE


@pytest.mark.parametrize("curve", [0, 1])
def test_noalloc_at_the_size_limit(curve):
    """n = 262144, the largest size the fixed array holds, on both curves, twice
    in a row, against the allocating entry point and the oracle; the free device
    memory is the same before and after the calls"""
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import make_workload
    lib = hs.load()
    ctx = hs.Context(0)
    try:
        n = MAX_POINTS
        w = make_workload(curve, n, 99 + curve, edge_fraction=0.01)
        d_u = torch.from_numpy(w.u.reshape(-1).copy()).cuda()
        d_pts = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
        d_sc = torch.from_numpy(w.scalars.reshape(-1).copy()).cuda()
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), n, d_pts.data_ptr())
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        pts = d_pts.cpu().numpy()
        idx = np.arange(0, n, 4099)
        assert (pts.reshape(n, 64)[idx] == oracle.map_to_curve(curve, w.u[idx].reshape(-1)).reshape(-1, 64)).all()
        want = oracle.msm_mt(curve, w.scalars, pts, oracle.default_threads())
        d_a = torch.zeros(120, dtype=torch.uint8, device="cuda")
        d_b = torch.zeros(120, dtype=torch.uint8, device="cuda")
        ctx.msm_device(curve, d_sc.data_ptr(), d_pts.data_ptr(), n, d_b.data_ptr(), HS_JAC51)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        b = ctx.compress(curve, d_b.cpu().numpy(), HS_JAC51).tobytes()
        assert b == want
        # the first call on a device may reserve the array (lazy module loading)
        assert _noalloc(lib, curve, d_sc, d_pts, n, d_a, HS_JAC51, None) == 0
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        outs = []
        for _ in range(2):
            d_a.zero_()
            torch.cuda.synchronize()
            assert _noalloc(lib, curve, d_sc, d_pts, n, d_a, HS_JAC51, None) == 0
            torch.cuda.synchronize()
            outs.append(d_a.cpu().numpy())
        assert torch.cuda.mem_get_info()[0] == free0
        for o in outs:
            assert ctx.compress(curve, o, HS_JAC51).tobytes() == want
    finally:
        ctx.close()
