"""Sharded MSM over the ranks of a torch.distributed process group.

An MSM is a sum, so it splits without any exchange on the data path: rank r
sums its contiguous slice of the (scalar, base) pairs on its own GPU and
returns one partial point; the only exchange is an all-gather of the G partial
points (64 bytes each, canonical affine) after which every rank adds them with
one G-term MSM of unit scalars on its GPU.  This is the decomposition the
reference's own callers use when they add per-chunk results with operator+
(include/helioselene_point.h:113-141, src/api_point.cpp:98-116).

The engine is anything with the Context.msm signature
``msm(curve, scalars, points, point_fmt, out_fmt) -> bytes``; on a GPU machine it
is a helioselene_gb300.Context.  Ranks that fail or leave before the gather
surface as ShardError on the others (the process group's own timeout bounds
the wait), never as a hang.
"""

from __future__ import annotations

from datetime import timedelta
from typing import List, Optional, Tuple

import numpy as np

from . import _lib as L


class ShardError(RuntimeError):
    """The partial-point exchange failed (a rank raised, left, or timed out)."""


def shard_range(n: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous slice [lo, hi) of n items for rank; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _as_rows(a, width: int) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.uint8)).reshape(-1)
    if arr.size % width:
        raise ValueError(f"buffer of {arr.size} bytes is not a multiple of {width}")
    return arr.reshape(-1, width)


def gather_partials(partial: bytes, group=None, timeout: Optional[timedelta] = None) -> List[bytes]:
    """All-gather one fixed-size byte record per rank, in rank order."""
    import torch
    import torch.distributed as dist

    rec = np.frombuffer(partial, dtype=np.uint8)
    backend = dist.get_backend(group)
    device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    mine = torch.from_numpy(rec.copy()).to(device)
    world = dist.get_world_size(group)
    outs = [torch.empty_like(mine) for _ in range(world)]
    try:
        work = dist.all_gather(outs, mine, group=group, async_op=True)
        if timeout is not None:
            work.wait(timeout)
        else:
            work.wait()
    except Exception as e:  # a peer raised, exited or never joined
        raise ShardError(f"partial-point gather failed on rank {dist.get_rank(group)}: {e}") from e
    return [o.cpu().numpy().tobytes() for o in outs]


def sharded_msm(engine, curve: int, scalars, points, point_fmt: int = L.FMT_AFFINE,
                out_fmt: int = L.FMT_COMPRESSED, group=None, timeout: Optional[timedelta] = None) -> bytes:
    """sum_i scalars[i] * points[i] over all ranks' data.

    Every rank passes the same full arrays (or at least its own slice at the
    right offsets); rank r computes the slice shard_range(n, G, r).  All ranks
    return the same result."""
    import torch.distributed as dist

    pb = L.FMT_BYTES[point_fmt]
    sc = _as_rows(scalars, 32)
    pts = _as_rows(points, pb)
    if sc.shape[0] != pts.shape[0]:
        raise ValueError("scalars and points differ in count")
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = shard_range(sc.shape[0], world, rank)
    partial = engine.msm(curve, sc[lo:hi], pts[lo:hi], point_fmt, L.FMT_AFFINE)
    parts = gather_partials(partial, group=group, timeout=timeout)
    return combine_partials(engine, curve, parts, out_fmt)


def combine_partials(engine, curve: int, parts: List[bytes], out_fmt: int = L.FMT_COMPRESSED) -> bytes:
    """Sum of canonical affine partial points (64 bytes each, identity = zeros)
    as one MSM with unit scalars, so the addition runs on the engine."""
    g = len(parts)
    ones = np.zeros((g, 32), np.uint8)
    ones[:, 0] = 1
    return engine.msm(curve, ones, np.frombuffer(b"".join(parts), np.uint8), L.FMT_AFFINE, out_fmt)
