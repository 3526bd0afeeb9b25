"""Rank bodies for the sharded-MSM tests (spawned processes, gloo on CPU).

The oracle stands in for the GPU engine here: these tests cover the host-side
split, exchange and failure handling, not the arithmetic."""

import os
import sys
import traceback
from datetime import timedelta
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

FMT_AFFINE, FMT_COMPRESSED = 2, 3


class OracleEngine:
    """Context.msm-shaped adapter over the oracle (test infrastructure only)."""

    def msm(self, curve, scalars, points, point_fmt, out_fmt):
        import oracle
        assert point_fmt == FMT_AFFINE
        if out_fmt == FMT_AFFINE:
            return oracle.msm_affine(curve, scalars, points)[1]
        assert out_fmt == FMT_COMPRESSED
        return oracle.msm(curve, scalars, points)


def _init(rank, world, port, timeout_s):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=timeout_s))
    return dist


def run_rank(rank, world, port, curve, n, seed, q):
    try:
        from conftest import oracle_inputs
        from helioselene_gb300.shard import sharded_msm
        dist = _init(rank, world, port, 60)
        sc, pts, _ = oracle_inputs(curve, n, seed=seed, edge_fraction=0.05)
        out = sharded_msm(OracleEngine(), curve, sc, pts, FMT_AFFINE, FMT_COMPRESSED)
        q.put((rank, "ok", out))
        dist.barrier()
        dist.destroy_process_group()
    except Exception:
        q.put((rank, "error", traceback.format_exc()))


def run_rank_failing(rank, world, port, curve, n, seed, q):
    """rank 1 fails before the exchange; rank 0 must get a ShardError, not hang"""
    try:
        from conftest import oracle_inputs
        from helioselene_gb300.shard import ShardError, sharded_msm
        dist = _init(rank, world, port, 15)
        sc, pts, _ = oracle_inputs(curve, n, seed=seed)
        if rank == 1:
            q.put((rank, "left", b""))
            q.close()
            q.join_thread()  # flush the message before leaving
            os._exit(3)  # leaves without joining the gather
        try:
            sharded_msm(OracleEngine(), curve, sc, pts, FMT_AFFINE, FMT_COMPRESSED, timeout=timedelta(seconds=15))
            q.put((rank, "no error", b""))
        except ShardError as e:
            q.put((rank, "shard_error", str(e).encode()))
    except Exception:
        q.put((rank, "error", traceback.format_exc()))
