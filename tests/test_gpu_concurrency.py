"""Host-thread concurrency and context options: contexts on several threads,
one context shared by threads (calls serialise on its lock), stream priority
and window-split changes between calls, and argument checks of the newer
entry points.  Results are compared bit for bit with the oracle."""

import threading

import numpy as np
import pytest

import oracle
from conftest import oracle_inputs

pytestmark = pytest.mark.gpu

HS_JAC51, HS_AFF51, HS_AFF, HS_COMPRESSED = 0, 1, 2, 3


def _cases(k):
    out = []
    for j in range(k):
        curve = j % 2
        n = [700, 3000, 20000, 70000][j % 4]
        sc, pts, _ = oracle_inputs(curve, n, seed=900 + j, edge_fraction=0.02)
        out.append((curve, sc, pts, oracle.msm(curve, sc, pts)))
    return out


def test_contexts_on_threads():
    import helioselene_gb300 as hs
    cases = _cases(8)
    results = [None] * len(cases)

    def work(i):
        with hs.Context(0) as c:
            for _ in range(2):
                curve, sc, pts, _ = cases[i]
                results[i] = c.msm(curve, sc, pts)

    ths = [threading.Thread(target=work, args=(i,)) for i in range(len(cases))]
    [t.start() for t in ths]
    [t.join() for t in ths]
    assert results == [w for *_, w in cases]


def test_shared_context_serialises(ctx):
    cases = _cases(6)
    results = [None] * len(cases)

    def work(i):
        curve, sc, pts, _ = cases[i]
        results[i] = ctx.msm(curve, sc, pts)

    ths = [threading.Thread(target=work, args=(i,)) for i in range(len(cases))]
    [t.start() for t in ths]
    [t.join() for t in ths]
    assert results == [w for *_, w in cases]


def test_priority_and_split_between_calls():
    import helioselene_gb300 as hs
    curve = 1
    n = (1 << 18) + 11
    sc, pts, _ = oracle_inputs(curve, 4000, seed=5)
    big_sc = np.tile(sc, ((n + 3999) // 4000, 1))[:n]
    big_pts = np.tile(np.frombuffer(pts, np.uint8).reshape(4000, 64), ((n + 3999) // 4000, 1))[:n]
    with hs.Context(0) as c:
        want = c.msm(curve, big_sc, big_pts)
        for prio in (True, False, True):
            c.set_priority(prio)
            for split in (0, 1 << 18, 1 << 10):
                c.set_split(split)
                assert c.msm(curve, big_sc, big_pts) == want
                assert c.msm_batch([(curve, big_sc[:5000], big_pts[:5000])])[0] == c.msm(curve, big_sc[:5000],
                                                                                          big_pts[:5000])


def test_argument_checks(ctx):
    import helioselene_gb300 as hs
    lib = hs.load()
    h = ctx.handle
    buf = np.zeros(1024, np.uint8)
    p = buf.ctypes.data
    assert lib.hs_decompress(h, 0, p, 1, p, HS_COMPRESSED, None) == hs._lib.HS_EINVAL   # not an output form
    assert lib.hs_decompress(h, 7, p, 1, p, HS_AFF, None) == hs._lib.HS_EINVAL          # no such curve
    assert lib.hs_scalar_mul(h, 0, None, p, HS_AFF, 1, p, HS_AFF) == hs._lib.HS_EINVAL
    assert lib.hs_scalar_mul(h, 0, p, p, 9, 1, p, HS_AFF) == hs._lib.HS_EINVAL          # no such point form
    assert lib.hs_scalar_mul(h, 0, p, p, HS_AFF, 0, p, HS_AFF) == hs._lib.HS_OK          # n = 0: nothing to do
    assert lib.hs_context_set_priority(None, 1) == hs._lib.HS_EINVAL
    assert lib.hs_context_set_split(None, 0) == hs._lib.HS_EINVAL
