"""Sharded MSM (one slice per rank, all-gather of partial points, one
unit-scalar MSM to add them): host-side split, exchange over gloo with
world_size 2, and a rank that leaves before the exchange.  The GPU test runs
the same decomposition with simulated shards on one device."""

import multiprocessing as mp
import socket

import numpy as np
import pytest

import oracle
from conftest import oracle_inputs
from helioselene_gb300.shard import combine_partials, shard_range


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n", [0, 1, 2, 5, 16, 1000, 1 << 20])
@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shard_range_partitions(n, world):
    spans = [shard_range(n, world, r) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    for (a, b), (c, d) in zip(spans, spans[1:]):
        assert b == c
    sizes = [b - a for a, b in spans]
    assert max(sizes) - min(sizes) <= 1


def test_shard_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _spawn(target, world, *args, timeout=120):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, *args, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        rank, status, payload = q.get(timeout=timeout)
        res[rank] = (status, payload)
    for p in procs:
        p.join(timeout=30)
        if p.is_alive():
            p.kill()
    return res


@pytest.mark.parametrize("curve", [0, 1])
def test_sharded_msm_two_ranks_gloo(curve):
    import _shard_worker as w
    n, seed = 300, 91 + curve
    res = _spawn(w.run_rank, 2, curve, n, seed)
    assert all(s == "ok" for s, _ in res.values()), res
    sc, pts, _ = oracle_inputs(curve, n, seed=seed, edge_fraction=0.05)
    want = oracle.msm(curve, sc, pts)
    assert res[0][1] == res[1][1] == want


def test_rank_leaving_before_exchange_raises_shard_error():
    import _shard_worker as w
    res = _spawn(w.run_rank_failing, 2, 0, 64, 5, timeout=90)
    assert res[1][0] == "left"
    assert res[0][0] == "shard_error", res[0]


def test_combine_partials_adds_points():
    import _shard_worker as w
    curve = 0
    sc, pts, _ = oracle_inputs(curve, 40, seed=3)
    parts = [oracle.msm_affine(curve, sc[a:b], pts[a:b])[1] for a, b in (shard_range(40, 4, r) for r in range(4))]
    parts.append(bytes(64))  # an empty shard contributes the identity
    assert combine_partials(w.OracleEngine(), curve, parts) == oracle.msm(curve, sc, pts)


@pytest.mark.gpu
@pytest.mark.parametrize("curve", [0, 1])
def test_simulated_shards_on_one_gpu(ctx, curve):
    """the GPU path for every shard and for the final addition, G = 1..8 shards"""
    n = 5000
    sc, pts, _ = oracle_inputs(curve, n, seed=17 + curve, edge_fraction=0.02)
    want = oracle.msm(curve, sc, pts)
    for g in (1, 2, 3, 8):
        parts = [ctx.msm(curve, sc[a:b], pts[a:b], 2, 2) for a, b in (shard_range(n, g, r) for r in range(g))]
        assert combine_partials(ctx, curve, parts) == want
