"""Window and accumulation autotuner for the batched and per-call MSM paths.

For every size class (powers of two from 2^6 to 2^20) it times, on the GPU, a
batch of MSMs of that size over candidate window widths c (a hill-climb that
starts from the previous class's best) and keeps the fastest; then, at that c,
the bucket accumulation form: 0, 1 or 2 batch-affine rounds (the wave of
pairwise additions that share one inversion, hs_context_set_batch_affine).
The table becomes the context's rules (hs_context_set_rule: c per class, and
the rounds of plans whose entries lie mostly in that class) and can be saved
to / loaded from a JSON cache keyed by device name.

The reference hard-codes its window by n (helios/src/x64/helios_msm_vartime.cpp:248-263)
and its autotune times only backends at n = 16 (src/dispatch.cpp:381-421); here
the choice is measured per size class on the device that will run it.
"""

from __future__ import annotations

import json
import time
from pathlib import Path
from typing import Dict, Iterable, Optional

import numpy as np

from . import _lib as L

DEFAULT_CANDIDATES = tuple(range(8, 17))


def _classes(n_min: int, n_max: int):
    k = max(1, int(np.floor(np.log2(max(1, n_min)))))
    while (1 << k) <= n_max:
        lo, hi = 1 << k, (1 << (k + 1)) - 1
        yield lo, hi
        k += 1


ROUND_CANDIDATES = (0, 1, 2)


def tune(ctx, curve: int, n_min: int = 64, n_max: int = 1 << 20, candidates: Iterable[int] = DEFAULT_CANDIDATES,
         points_per_class: int = 1 << 20, reps: int = 3, seed: int = 1) -> Dict[str, dict]:
    """Return {"lo-hi": {"c": c, "rounds": r}} for each size class, measured with
    batched device MSMs.

    Window candidates are walked outward from the best of the previous size
    class (the optimum grows with n), stopping once two neighbours in a row are
    slower; the accumulation rounds are then timed at the chosen c (a batch
    below the accumulation's entry threshold runs XYZZ whatever the rounds, so
    its class keeps 0)."""
    import torch

    from .workload import ORDER, random_field_bytes, random_scalars
    rng = np.random.default_rng(seed)
    table = {}
    prev = 8
    stream = torch.cuda.ExternalStream(ctx.stream)
    for lo, hi in _classes(n_min, n_max):
        n = lo + (hi - lo) // 2
        count = max(1, min(256, points_per_class // n))
        total = n * count
        d_u = torch.from_numpy(random_field_bytes(rng, total).reshape(-1)).cuda()
        d_pts = torch.empty(total * 64, dtype=torch.uint8, device="cuda")
        d_sc = torch.from_numpy(random_scalars(rng, total, ORDER[curve]).reshape(-1)).cuda()
        d_out = torch.empty(count * 120, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), total, d_pts.data_ptr())
        sizes = [n] * count
        cands = sorted(set(candidates))
        timed = {}

        def measure(c, rounds=0):
            if (c, rounds) not in timed:
                ctx.set_window(curve, 0, 0, 0)
                ctx.set_window(curve, 1, 1 << 31, c, rounds)
                ctx.msm_batch_device(curve, sizes, d_sc.data_ptr(), d_pts.data_ptr(), d_out.data_ptr())
                stream.synchronize()
                ts = []
                for _ in range(reps):
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    ctx.msm_batch_device(curve, sizes, d_sc.data_ptr(), d_pts.data_ptr(), d_out.data_ptr())
                    b.record(stream)
                    stream.synchronize()
                    ts.append(a.elapsed_time(b))
                timed[(c, rounds)] = min(ts)
            return timed[(c, rounds)]

        start = min(cands, key=lambda c: abs(c - prev)) if table else cands[0]
        best_c = start
        for direction in (+1, -1):
            worse = 0
            c = start + direction
            while cands[0] <= c <= cands[-1] and worse < 2:
                if measure(c) < measure(best_c):
                    best_c, worse = c, 0
                else:
                    worse += 1
                c += direction
        measure(start)
        prev = best_c
        best_r = min(ROUND_CANDIDATES, key=lambda r: measure(best_c, r))
        table[f"{lo}-{hi}"] = {"c": best_c, "rounds": best_r}
        del d_u, d_pts, d_sc, d_out
    ctx.set_window(curve, 0, 0, 0)
    return table


def apply(ctx, curve: int, table: Dict[str, object]) -> None:
    """install a table: entries {"c", "rounds"} (or a bare window width)"""
    ctx.set_window(curve, 0, 0, 0)
    for key, v in table.items():
        lo, hi = (int(x) for x in key.split("-"))
        if isinstance(v, dict):
            ctx.set_window(curve, lo, hi, int(v["c"]), int(v.get("rounds", -1)))
        else:
            ctx.set_window(curve, lo, hi, int(v))


def load_or_tune(ctx, cache: Optional[Path] = None, n_max: int = 1 << 20, **kw) -> dict:
    """Tables for both curves from the cache (matching device) or freshly tuned."""
    import torch
    dev = torch.cuda.get_device_name(ctx.device)
    data = {}
    if cache and Path(cache).exists():
        try:
            data = json.loads(Path(cache).read_text())
        except (OSError, ValueError):
            data = {}
    entry = data.get(dev)
    stale = entry and not all(isinstance(v, dict) for k in ("helios", "selene") for v in entry.get(k, {}).values())
    if not entry or stale or entry.get("n_max", 0) < n_max:
        t0 = time.time()
        entry = {"n_max": n_max, "helios": tune(ctx, L.HELIOS, n_max=n_max, **kw),
                 "selene": tune(ctx, L.SELENE, n_max=n_max, **kw), "seconds": round(time.time() - t0, 2)}
        data[dev] = entry
        if cache:
            try:
                Path(cache).write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
            except OSError:
                pass
    apply(ctx, L.HELIOS, entry["helios"])
    apply(ctx, L.SELENE, entry["selene"])
    return entry
