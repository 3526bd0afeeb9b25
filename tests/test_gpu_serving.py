"""Continuous-batching server: results against the oracle, identical alone and in
the mix, resident pool + fresh bases, HBM-budget deferral, bad requests refused."""

import numpy as np
import pytest

import oracle
from conftest import oracle_inputs

pytestmark = pytest.mark.gpu


def make_requests(rng, pools, count, pool_n):
    reqs = []
    for i in range(count):
        curve = i % 2  # alternating cycle layers
        n = int(np.exp(rng.uniform(np.log(2), np.log(6000))))
        n_pool = int(rng.integers(0, n + 1))
        n_fresh = n - n_pool
        idx = rng.integers(0, pool_n, n_pool).astype(np.uint32)
        sc, fresh, _ = oracle_inputs(curve, max(1, n_fresh), seed=10000 + i)
        fresh = fresh[:n_fresh]
        from helioselene_gb300.workload import ORDER, random_scalars
        scal = random_scalars(rng, n, ORDER[curve])
        pts = np.concatenate([pools[curve][idx], fresh]) if n else np.zeros((0, 64), np.uint8)
        reqs.append({"curve": curve, "scalars": scal, "idx": idx, "fresh": fresh,
                     "want": oracle.msm(curve, scal, pts)})
    return reqs


@pytest.fixture(scope="module")
def pools():
    out = {}
    for curve in (0, 1):
        _, pts, _ = oracle_inputs(curve, 4096, seed=777 + curve)
        out[curve] = pts
    return out


def test_server_mixed_stream(pools):
    import helioselene_gb300 as hs
    rng = np.random.default_rng(1)
    reqs = make_requests(rng, pools, 60, 4096)
    with hs.Server(0, slots=3) as srv:
        for c in (0, 1):
            srv.set_pool(c, pools[c])
        tickets = [srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]) for r in reqs]
        got = [srv.wait(t)[0] for t in tickets]
        st = srv.stats()
    bad = [i for i, (g, r) in enumerate(zip(got, reqs)) if g != r["want"]]
    assert not bad, f"mismatches {bad[:8]}"
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] < len(reqs)  # requests were batched together


def test_same_alone_and_in_the_mix(pools):
    import helioselene_gb300 as hs
    rng = np.random.default_rng(2)
    reqs = make_requests(rng, pools, 24, 4096)
    with hs.Server(0, slots=2) as srv:
        for c in (0, 1):
            srv.set_pool(c, pools[c])
        alone = []
        for r in reqs:  # one at a time: each is a batch of one
            alone.append(srv.wait(srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]))[0])
        tickets = [srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]) for r in reqs]
        mixed = [srv.wait(t)[0] for t in tickets]
    assert alone == mixed
    assert alone == [r["want"] for r in reqs]


def test_window_rules_apply_to_every_slot(pools):
    """hs_server_set_window: every window width the slots may be given yields the
    same results; bad rules are refused"""
    import helioselene_gb300 as hs
    from helioselene_gb300._lib import HsError
    rng = np.random.default_rng(3)
    reqs = make_requests(rng, pools, 16, 4096)
    with hs.Server(0, slots=2) as srv:
        for c in (0, 1):
            srv.set_pool(c, pools[c])
        for w in (5, 9, 13):
            for c in (0, 1):
                srv.set_window(c, 0, 0, 0)
                srv.set_window(c, 1, 1 << 20, w)
            tickets = [srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]) for r in reqs]
            got = [srv.wait(t)[0] for t in tickets]
            assert got == [r["want"] for r in reqs], f"window {w}"
        for bad in ((2, 0, 10, 8), (0, 10, 5, 8), (0, 0, 10, 3), (0, 0, 10, 21)):
            with pytest.raises(HsError):
                srv.set_window(*bad)


def test_budget_defers_but_completes(pools):
    import helioselene_gb300 as hs
    rng = np.random.default_rng(3)
    reqs = make_requests(rng, pools, 20, 4096)
    # a budget of ~one small batch: the scheduler must hold launches back until memory frees up
    with hs.Server(0, slots=4, hbm_budget=48 << 20, max_batch_msms=4) as srv:
        for c in (0, 1):
            srv.set_pool(c, pools[c])
        tickets = [srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]) for r in reqs]
        got = [srv.wait(t)[0] for t in tickets]
        st = srv.stats()
    assert got == [r["want"] for r in reqs]
    assert st["peak_bytes"] > 0


def test_bad_requests_are_refused(pools):
    import helioselene_gb300 as hs
    with hs.Server(0, slots=1, max_batch_points=1000) as srv:
        srv.set_pool(0, pools[0])
        sc = np.zeros((4, 32), np.uint8)
        with pytest.raises(hs.HsError) as e:
            srv.submit(0, sc, np.array([0, 1, 2, 99999], np.uint32))  # index outside the pool
        assert e.value.status == -1
        with pytest.raises(hs.HsError) as e:
            srv.submit(0, np.zeros((2000, 32), np.uint8), np.zeros(2000, np.uint32))  # above the batch cap
        assert e.value.status == -6
        t = srv.submit(0, sc, np.array([0, 1, 2, 3], np.uint32))
        assert srv.wait(t)[0] == bytes(32)  # zero scalars -> identity


@pytest.mark.parametrize("window", [0, 6, 12, 16])
def test_pool_table_widths_and_part_shapes(pools, window):
    """the pool as a table of window multiples (pool-only requests as fixed-base
    MSMs over indexed rows, batched apart from the requests with fresh bases), or
    gathered (window 0): every request shape -- pooled only, fresh only, both,
    empty, repeated and identity-cancelling indices -- matches the oracle, in
    the mix and alone"""
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import ORDER, random_scalars
    rng = np.random.default_rng(40 + window)
    reqs = make_requests(rng, pools, 30, 4096)
    for curve in (0, 1):
        for n_pool, n_fresh in ((700, 0), (0, 300), (0, 0), (1, 0), (5000, 20)):
            idx = rng.integers(0, 4096, n_pool).astype(np.uint32)
            if n_pool >= 700:
                idx[: n_pool // 4] = 17  # one pool point many times: doubling and cancelling cases
            _, fresh, _ = oracle_inputs(curve, max(1, n_fresh), seed=90 + n_fresh)
            fresh = fresh[:n_fresh]
            scal = random_scalars(rng, n_pool + n_fresh, ORDER[curve])
            if n_pool >= 700:
                # s and order - s on the same pool point cancel
                s0 = int.from_bytes(scal[0].tobytes(), "little")
                scal[1] = np.frombuffer((ORDER[curve] - s0).to_bytes(32, "little"), np.uint8)
                idx[1] = idx[0]
            pts = np.concatenate([pools[curve][idx], fresh]) if n_pool + n_fresh else np.zeros((0, 64), np.uint8)
            reqs.append({"curve": curve, "scalars": scal, "idx": idx, "fresh": fresh,
                         "want": oracle.msm(curve, scal, pts)})
    with hs.Server(0, slots=3) as srv:
        for c in (0, 1):
            srv.set_pool_window(c, window)
            srv.set_pool(c, pools[c])
        tickets = [srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]) for r in reqs]
        got = [srv.wait(t)[0] for t in tickets]
        alone = [srv.wait(srv.submit(r["curve"], r["scalars"], r["idx"], r["fresh"]))[0] for r in reqs[-10:]]
        st = srv.stats()
    bad = [i for i, (g, r) in enumerate(zip(got, reqs)) if g != r["want"]]
    assert not bad, f"mismatches {bad[:8]}"
    assert alone == got[-10:]
    assert st["failed"] == 0


def test_pool_window_refused_outside_range(pools):
    import helioselene_gb300 as hs
    with hs.Server(0, slots=1) as srv:
        for bad in ((2, 12), (0, 3), (0, 17), (1, -1)):
            with pytest.raises(hs.HsError):
                srv.set_pool_window(*bad)
