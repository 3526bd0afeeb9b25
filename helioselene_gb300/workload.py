"""Seeded synthetic MSM workloads with the shapes of the benchmark configurations.

* scalars: uniform in [0, order) (32 random bytes, bit 255 cleared, values
  >= order redrawn), the distribution HeliosScalar::from_bytes accepts
  (src/api_scalar.cpp:46-67);
* bases: simplified-SWU images of uniform field elements (the reference's
  HeliosPoint::map_to_curve, src/api_point.cpp:146-151) -- this module only
  draws the u values, the map itself runs on the GPU (hs_map_to_curve);
* edge slices (1% in total when requested): zero scalars, scalar = order-1,
  one base repeated with one equal scalar (every window then hits the bucket
  doubling case), and scalars with only the top window nonzero.

The batched stream (1024 MSMs of log-uniform sizes, either curve) and the
serving mixture are generated here too, so that the parity tests check the
exact inputs the benchmark times.

There is no public dataset for this path; these seeded inputs stand in for it.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ._lib import HELIOS, SELENE

# seed of the benchmark's workloads (each configuration adds its own offset)
BENCH_SEED = 0x48454C494F53

P = 2**255 - 19
Q = 2**255 - 85737960593035654572250192257530476641
ORDER = {HELIOS: Q, SELENE: P}     # Helios has order q, Selene has order p (the cycle)
FIELD = {HELIOS: P, SELENE: Q}


def _order_words(order: int) -> np.ndarray:
    return np.array([(order >> (64 * i)) & (2**64 - 1) for i in range(4)], dtype=np.uint64)


def below(words: np.ndarray, bound: int) -> np.ndarray:
    """Rows of (n,4) little-endian u64 words that are < bound."""
    b = _order_words(bound)
    lt = np.zeros(words.shape[0], bool)
    eq = np.ones(words.shape[0], bool)
    for i in (3, 2, 1, 0):
        lt |= eq & (words[:, i] < b[i])
        eq &= words[:, i] == b[i]
    return lt


def random_scalars(rng: np.random.Generator, n: int, order: int) -> np.ndarray:
    """(n, 32) uint8, uniform in [0, order)."""
    out = np.empty((n, 4), np.uint64)
    todo = np.arange(n)
    while todo.size:
        w = rng.integers(0, 2**64, size=(todo.size, 4), dtype=np.uint64)
        w[:, 3] &= np.uint64(0x7FFFFFFFFFFFFFFF)
        ok = below(w, order)
        out[todo[ok]] = w[ok]
        todo = todo[~ok]
    return out.view(np.uint8).reshape(n, 32)


def random_field_bytes(rng: np.random.Generator, n: int) -> np.ndarray:
    """(n, 32) uint8 u values for the SWU map (bit 255 cleared, as fp_frombytes masks it)."""
    u = rng.integers(0, 256, size=(n, 32), dtype=np.uint8)
    u[:, 31] &= 0x7F
    return u


def int_to_bytes32(v: int) -> np.ndarray:
    return np.frombuffer(v.to_bytes(32, "little"), dtype=np.uint8)


@dataclass
class Workload:
    curve: int
    n: int
    scalars: np.ndarray      # (n, 32) uint8
    u: np.ndarray            # (n, 32) uint8, bases = map_to_curve(u)
    edge: dict               # name -> index array of the edge slices


def make_workload(curve: int, n: int, seed: int, edge_fraction: float = 0.0) -> Workload:
    rng = np.random.default_rng(seed)
    order = ORDER[curve]
    scalars = random_scalars(rng, n, order)
    u = random_field_bytes(rng, n)
    edge = {}
    k = int(n * edge_fraction / 4)
    if k > 0:
        idx = rng.permutation(n)[: 4 * k].reshape(4, k)
        zero, top1, rep, topw = idx
        scalars[zero] = 0
        scalars[top1] = int_to_bytes32(order - 1)
        # one base repeated with one equal scalar: forces the doubling case in every window
        u[rep] = u[rep[0]]
        scalars[rep] = scalars[rep[0]]
        # only bits 240..254 set (random < 2^15, shifted up), kept below the order
        hi = rng.integers(1, 2**15, size=k, dtype=np.uint64)
        top = np.zeros((k, 4), np.uint64)
        top[:, 3] = hi << np.uint64(48)
        ok = below(top, order)
        top[~ok, 3] = np.uint64(1) << np.uint64(48)
        scalars[topw] = top.view(np.uint8).reshape(k, 32)
        edge = {"zero": zero, "order_minus_1": top1, "repeated": rep, "top_window": topw}
    return Workload(curve, n, scalars, u, edge)


def batched_stream(seed: int = BENCH_SEED + 3, count: int = 1024) -> dict:
    """The batched configuration: `count` independent MSMs, sizes log-uniform in
    [64, 65536], curve Helios or Selene with probability 1/2, uniform scalars and
    SWU bases.  Returns {"sizes", "curves", HELIOS: group, SELENE: group}, a
    group being {"idx": MSM indices, "sizes": list, "u": (total, 32) SWU inputs,
    "scalars": (total, 32)}, the MSMs of a group back to back."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(64), np.log(65536), count)).astype(np.int64)
    curves = rng.integers(0, 2, count)
    out = {"sizes": sizes, "curves": curves}
    for curve in (HELIOS, SELENE):
        idx = np.nonzero(curves == curve)[0]
        sz = [int(sizes[i]) for i in idx]
        total = sum(sz)
        u = random_field_bytes(rng, total)
        sc = random_scalars(rng, total, ORDER[curve])
        out[curve] = {"idx": idx, "sizes": sz, "u": u, "scalars": sc}
    return out


def serving_sizes(rng: np.random.Generator, count: int) -> np.ndarray:
    """Request sizes of the serving mixture: 70% log-uniform [256, 4096], 25%
    log-uniform [4096, 65536], 5% exactly 2^18."""
    u = rng.random(count)
    n = np.where(u < 0.70, np.exp(rng.uniform(np.log(256), np.log(4096), count)),
                 np.where(u < 0.95, np.exp(rng.uniform(np.log(4096), np.log(65536), count)), 2.0**18))
    return n.astype(np.int64)
