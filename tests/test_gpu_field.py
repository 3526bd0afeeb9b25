"""Device field arithmetic (F_p, F_q in eight 32-bit limbs) against Python integers.
Inputs cover the whole 256-bit range, including the weak-reduction edges
(m-1, m, 2m, 2m+c-1 = 2^256-1) where the fold and the canonical reduction
have their corner cases."""

import random

import numpy as np
import pytest

import pyref

pytestmark = pytest.mark.gpu

MODULI = {0: pyref.P, 1: pyref.Q}


def edge_values(m):
    c = 2**256 % m
    base = [0, 1, 2, 19, 38, m - 1, m, m + 1, 2 * m - 1, 2 * m, 2 * m + 1, 2**256 - 1, 2**256 - c, 2**255,
            2**255 - 1, c, c - 1, 2**128, 2**224 - 1]
    return [v % 2**256 for v in base]


def to_bytes(vals):
    return np.frombuffer(b"".join(v.to_bytes(32, "little") for v in vals), np.uint8)


def from_bytes(arr):
    b = arr.tobytes()
    return [int.from_bytes(b[32 * i:32 * i + 32], "little") for i in range(len(b) // 32)]


@pytest.mark.parametrize("field", [0, 1])
def test_field_ops_match_integers(ctx, field):
    m = MODULI[field]
    rng = random.Random(field + 17)
    edges = edge_values(m)
    a = edges + [rng.getrandbits(256) for _ in range(20000)]
    b = list(reversed(edges)) + [rng.getrandbits(256) for _ in range(20000)]
    # all pairs of edge values too
    for x in edges:
        for y in edges:
            a.append(x)
            b.append(y)
    A, B = to_bytes(a), to_bytes(b)
    checks = {
        0: [(x * y) % m for x, y in zip(a, b)],
        1: [(x * x) % m for x in a],
        2: [(x + y) % m for x, y in zip(a, b)],
        3: [(x - y) % m for x, y in zip(a, b)],
        4: [x % m for x in a],
        6: [(-x) % m for x in a],
    }
    for op, want in checks.items():
        got = from_bytes(ctx.field_op(field, op, A, B))
        bad = [i for i, (g, w) in enumerate(zip(got, want)) if g != w]
        assert not bad, f"field {field} op {op}: {len(bad)} mismatches, first a={a[bad[0]]:#x} b={b[bad[0]]:#x}"
    inv_in = a[:3000]
    got = from_bytes(ctx.field_op(field, 5, to_bytes(inv_in)))
    for x, g in zip(inv_in, got):
        assert g == (pow(x, m - 2, m) if x % m else 0)


@pytest.mark.parametrize("field", [0, 1])
def test_chained_products_stay_reduced(ctx, field):
    """long chains of weakly-reduced products: x_{k+1} = x_k^2 * x_k"""
    m = MODULI[field]
    rng = random.Random(5)
    x = [rng.getrandbits(256) for _ in range(512)] + [2**256 - 1, m - 1, 2 * m]
    xs = [v % m for v in x]
    X = to_bytes(x)
    for _ in range(20):
        S = ctx.field_op(field, 1, X)
        X = ctx.field_op(field, 0, S, X)
        xs = [(v * v % m) * v % m for v in xs]
    assert from_bytes(X) == xs


@pytest.mark.parametrize("field", [0, 1])
def test_lane_sliced_field_matches_integers(ctx, field):
    """the window combination's field form (radix-2^26 limbs across a warp's
    lanes, column products, carry steps and folds by 2^260 mod m) against
    Python integers, on the weak-reduction edges and random values"""
    m = MODULI[field]
    rng = random.Random(field + 71)
    edges = edge_values(m)
    a = edges + [rng.getrandbits(256) for _ in range(4000)] + [2**256 - 1 - rng.getrandbits(20) for _ in range(500)]
    b = list(reversed(edges)) + [rng.getrandbits(256) for _ in range(4000)] + [2**256 - 1 - rng.getrandbits(20)
                                                                             for _ in range(500)]
    for x in edges:
        for y in edges:
            a.append(x)
            b.append(y)
    A, B = to_bytes(a), to_bytes(b)
    checks = {
        7: [(x * y) % m for x, y in zip(a, b)],
        8: [((x - y) * (x + y)) % m for x, y in zip(a, b)],
        9: [pow(x, 2**32, m) for x in a],
        10: [x % m for x in a],
    }
    for op, want in checks.items():
        got = from_bytes(ctx.field_op(field, op, A, B))
        bad = [i for i, (g, w) in enumerate(zip(got, want)) if g != w]
        assert not bad, f"field {field} op {op}: {len(bad)} mismatches, first a={a[bad[0]]:#x} b={b[bad[0]]:#x}"
