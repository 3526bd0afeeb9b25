"""Batch-affine bucket accumulation (hs_context_set_batch_affine): rounds of
pairwise affine additions that share one inversion per 2048 additions, then an
XYZZ fold.  Every result is compared bit for bit with the oracle and with the
XYZZ accumulation of every entry (rounds = 0), on the cases the affine formula
treats apart: equal bases in a bucket (doubling), a base and its negation
(the identity), identity bases, lists of odd length (a carried item), empty
and one-entry buckets, and one bucket of thousands of entries."""

import numpy as np
import pytest

import oracle
import pyref
from conftest import oracle_inputs

pytestmark = pytest.mark.gpu

HS_AFF, HS_COMPRESSED = 2, 3


def _neg(curve, pts, i):
    F = pyref.CURVES["helios" if curve == 0 else "selene"].F
    y = int.from_bytes(pts[i, 32:].tobytes(), "little")
    out = pts[i].copy()
    out[32:] = np.frombuffer(((F - y) % F).to_bytes(32, "little"), np.uint8)
    return out


@pytest.fixture
def ba_ctx(ctx):
    yield ctx
    ctx.default_batch_affine()


@pytest.mark.parametrize("curve", [0, 1])
@pytest.mark.parametrize("n", [1, 2, 3, 17, 300, 4096, 20000])
def test_forced_rounds_match_oracle(ba_ctx, curve, n):
    """every round count forced on small plans (min_entries = 0), edge slices mixed in"""
    sc, pts, _ = oracle_inputs(curve, n, seed=n + 5 * curve, edge_fraction=0.08 if n >= 100 else 0.0)
    want = oracle.msm(curve, sc, pts)
    for rounds in (1, 2, 3):
        ba_ctx.set_batch_affine(rounds, 0)
        assert ba_ctx.msm(curve, sc, pts) == want, f"rounds={rounds}"


@pytest.mark.parametrize("curve", [0, 1])
def test_doubling_cancellation_and_identity_cases(ba_ctx, curve):
    n = 3000
    sc, pts, _ = oracle_inputs(curve, n, seed=71 + curve)
    pts = pts.copy()
    sc = sc.copy()
    pts[10:40] = 0                      # identity bases
    for i in range(100, 160):           # P and -P with equal scalars: pairs that cancel
        pts[i + 60] = _neg(curve, pts, i)
        sc[i + 60] = sc[i]
    pts[300:400] = pts[299]             # one base repeated with one scalar: doublings, then sums of equal sums
    sc[300:400] = sc[299]
    pts[500:520] = pts[499]             # a repeated base with different scalars
    sc[700:800] = 0                     # zero scalars
    sc[900:910] = 0xFF                  # unreduced scalars
    want = oracle.msm(curve, sc, pts)
    for rounds in (0, 1, 2, 3):
        ba_ctx.set_batch_affine(rounds, 0)
        assert ba_ctx.msm(curve, sc, pts) == want, f"rounds={rounds}"
    # everything cancels: s P + s (-P) for many P
    m = 512
    two = np.concatenate([sc[:m], sc[:m]])
    pm = np.concatenate([pts[1000:1000 + m], np.stack([_neg(curve, pts, i) for i in range(1000, 1000 + m)])])
    for rounds in (1, 2, 3):
        ba_ctx.set_batch_affine(rounds, 0)
        assert ba_ctx.msm(curve, two, pm) == bytes(32), f"rounds={rounds}"
        assert ba_ctx.msm(curve, np.zeros_like(sc), pts) == bytes(32)


@pytest.mark.parametrize("curve", [0, 1])
def test_default_rule_at_2p20_against_xyzz_and_oracle(ba_ctx, curve):
    """n = 2^20 with the 1% edge slices (the headline size): one, two and three
    rounds and the XYZZ path, split and unsplit, and the library default"""
    from helioselene_gb300.workload import make_workload
    n = 1 << 20
    w = make_workload(curve, n, seed=2024 + curve, edge_fraction=0.01)
    pts = ba_ctx.map_to_curve(curve, w.u, HS_AFF)
    want = oracle.msm_mt(curve, w.scalars, pts, oracle.default_threads())
    try:
        for split in (0, 1 << 18):
            ba_ctx.set_split(split)
            for rounds in (0, 1, 2, 3):
                ba_ctx.set_batch_affine(rounds, 1 << 21)
                assert ba_ctx.msm(curve, w.scalars, pts) == want, f"rounds={rounds} split={split}"
            ba_ctx.default_batch_affine()
            assert ba_ctx.msm(curve, w.scalars, pts) == want, f"default split={split}"
    finally:
        ba_ctx.set_split(1 << 18)


def test_batched_plan_with_rounds(ba_ctx):
    """a batch of MSMs of mixed sizes and both curves through one plan per curve"""
    items, wants = [], []
    rng = np.random.default_rng(3)
    for i, n in enumerate([5, 900, 1, 40000, 3000, 77777, 2]):
        curve = int(rng.integers(0, 2))
        sc, pts, _ = oracle_inputs(curve, n, seed=900 + i, edge_fraction=0.04 if n >= 100 else 0.0)
        items.append((curve, sc, pts))
        wants.append(oracle.msm(curve, sc, pts))
    for rounds in (1, 2, 3):
        ba_ctx.set_batch_affine(rounds, 0)
        got = ba_ctx.msm_batch(items)
        assert got == wants, f"rounds={rounds}"


@pytest.mark.parametrize("curve", [0, 1])
def test_rounds_from_size_class_rules(ba_ctx, curve):
    """window rules that name batch-affine rounds (what the autotuner installs):
    a batch whose entries lie mostly in one class takes that class's rounds"""
    items, wants = [], []
    for i, n in enumerate([70000, 3000, 90000, 17]):
        sc, pts, _ = oracle_inputs(curve, n, seed=4000 + i, edge_fraction=0.02 if n >= 100 else 0.0)
        items.append((curve, sc, pts))
        wants.append(oracle.msm(curve, sc, pts))
    try:
        for rounds in (0, 1, 2, 3):
            ba_ctx.set_window(curve, 0, 0, 0)
            ba_ctx.set_window(curve, 1, 4095, 9, 0)
            ba_ctx.set_window(curve, 4096, 1 << 20, 12, rounds)
            ba_ctx.set_batch_affine(0, 0, curve)  # the rules' rounds, not the curve setting, decide
            assert ba_ctx.msm_batch(items) == wants, f"rounds={rounds}"
            assert ba_ctx.msm(curve, items[2][1], items[2][2]) == wants[2], f"single, rounds={rounds}"
    finally:
        ba_ctx.set_window(curve, 0, 0, 0)


@pytest.mark.parametrize("curve", [0, 1])
def test_fixed_base_commitments_with_rounds(ba_ctx, curve):
    """fixed-base commitments (every window of every generator into one set of
    buckets, so buckets of thousands of entries) with the rounds forced on"""
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import ORDER, random_scalars
    n, count = 500, 5
    _, gens, _ = oracle_inputs(curve, n + 1, seed=61 + curve)
    H, G = gens[n], gens[:n]
    rng = np.random.default_rng(17 + curve)
    vals = random_scalars(rng, count * n, ORDER[curve]).reshape(count, n, 32)
    vals[1, :100] = vals[1, 0]          # repeated scalars on distinct generators
    vals[2] = 0
    blinds = random_scalars(rng, count, ORDER[curve])
    want = [oracle.pedersen(curve, blinds[j], H, vals[j], G) for j in range(count)]
    fb = hs.FixedBase(ba_ctx, curve, G, H=H, window=12)
    try:
        for rounds in (0, 1, 2, 3):
            ba_ctx.set_batch_affine(rounds, 0, curve)
            assert fb.commit(vals, blinds) == want, f"rounds={rounds}"
    finally:
        fb.close()


@pytest.mark.parametrize("curve", [0, 1])
def test_default_forms_restored(ba_ctx, curve):
    """rounds = -1 restores the library's per-kind defaults (host-input MSMs and
    fixed-base commitments: none on Helios, one on Selene; device MSMs: one),
    and every kind of plan still matches the oracle"""
    import helioselene_gb300 as hs
    from helioselene_gb300._lib import HsError
    n = 300000
    sc, pts, _ = oracle_inputs(curve, n, seed=808 + curve, edge_fraction=0.01)
    want = oracle.msm_mt(curve, sc, pts, oracle.default_threads())
    ba_ctx.set_batch_affine(3, 0, curve)
    assert ba_ctx.msm(curve, sc, pts) == want
    ba_ctx.set_batch_affine(-1, 0, curve)
    assert ba_ctx.msm(curve, sc, pts) == want
    assert ba_ctx.msm_batch([(curve, sc, pts)])[0] == want
    with pytest.raises(HsError):
        ba_ctx.set_batch_affine(-2, 0, curve)
    with pytest.raises(HsError):
        ba_ctx.set_batch_affine(4, 0, curve)
