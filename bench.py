"""Benchmark: Helios + Selene vartime MSM at n = 2^20, points per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n N]

One step = one Helios MSM and one Selene MSM of n = 2^20 points each (uniform
scalars mod the group order, SWU bases, 1% edge slices), on inputs already
resident in device memory.  The K timed steps are issued back to back with no
L2 flush between them: one step's inputs and workspaces (2 x 96 MiB of
scalars and bases alone) exceed the 129 MB L2.  `value` = 2n points / step
time, max over ranks.  The isolated-step latency beside it flushes L2 (256 MiB
memset) before each of its steps.
`e2e` = the same metric through the reference-facing call with host buffers:
hs_msm with the reference's helios_jacobian records (pinned host memory),
host-to-device copies, the device MSM, and the result read back, every step.

Multi-GPU: the MSMs of this workload do not shard across GPUs in this
design (replicas only): under torchrun every rank runs the same workload on
its own GPU and `value` sums the points of all ranks over the slowest rank's
time.

--impl reference times the reference's CPU algorithm (the oracle's C
restatement of helioselene's Pippenger, all host threads) on the same
workload, rank 0 only.
"""

from __future__ import annotations

import argparse
import contextlib
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MSM points/sec at n=2^20 (both curves, bit-exact); batched-serving MSMs/sec + p50/p99 vs plain"
WORKLOAD = ("Helios + Selene vartime Pippenger MSM, n=2^20 each; scalars uniform mod order; "
            "SWU-derived affine bases; 1% edge slices (zero, order-1, repeated base, top-window-only)")
from helioselene_gb300.workload import BENCH_SEED as SEED  # noqa: E402
IMAD_PER_MODMUL = {0: 144, 1: 232}  # F_p, F_q: 2 IMAD per 32x32->64 product
# dram__bytes_read.sum + dram__bytes_write.sum of the bucket-accumulation phase of
# one MSM at n = 2^20 (Helios, Selene), from ncu --set full captures of this
# workload, by accumulation form (batch-affine rounds): 0 is k_accumulate, 1 is
# k_ba_pairs + k_ba_invert + k_ba_finish + k_accumulate_level
ACC_TRAFFIC = {
    0: {"bytes": (477.2e6, 497.5e6), "capture": ("2026-12-04, commit 14d24da, k_accumulate",) * 2},
    1: {"bytes": (2916.1e6, 2941.9e6),
        "capture": ("2026-12-04, commit f0491f5, k_ba_pairs + k_ba_invert + k_ba_finish + k_accumulate_level",
                    "2026-12-04, commit d2e236f, k_ba_pairs + k_ba_invert + k_ba_finish + k_accumulate_level")},
    2: {"bytes": (None, 4316.5e6),
        "capture": (None, "2026-12-04, commit f0491f5, two rounds of k_ba_pairs + k_ba_invert + k_ba_finish, "
                          "then k_accumulate_level")},
}
DEFAULT_BA_ROUNDS = (1, 2)  # the library's default accumulation form of device-resident MSMs (Helios, Selene)
HOST_BA_ROUNDS = (0, 1)     # ... and of single MSMs from host buffers
SPLIT_DEFAULT = 1 << 18  # the library's window-split threshold for single MSMs


@contextlib.contextmanager
def no_python_gc():
    """Python's cyclic garbage collector paused around a host-timed loop: a full
    collection in a process holding torch's objects takes 10-20 ms and landed in
    about one run in six as a single slow step.  The library's calls are native
    code; the pause is the harness's, not theirs."""
    gc.collect()
    gc.freeze()
    gc.disable()
    try:
        yield
    finally:
        gc.enable()
        gc.unfreeze()


def host_cpu_state() -> dict:
    """The process's CPU time and its cgroup's CPU quota and throttling counters
    (cgroup v2 or v1), for reading host-timed loops: a cgroup that exhausts its
    quota in a scheduling period has every thread descheduled until the period
    ends (up to 100 ms by default)."""
    out = {"process_cpu_s": time.process_time(), "wall_s": time.perf_counter()}
    try:  # time the hypervisor ran something else on this machine's CPUs (all CPUs, USER_HZ ticks)
        with open("/proc/stat") as f:
            fields = f.readline().split()
        if fields[0] == "cpu" and len(fields) > 8:
            out["steal_ms"] = int(fields[8]) * 1e3 / os.sysconf("SC_CLK_TCK")
    except (OSError, ValueError):
        pass
    for stat, quota in (("/sys/fs/cgroup/cpu.stat", "/sys/fs/cgroup/cpu.max"),
                        ("/sys/fs/cgroup/cpu,cpuacct/cpu.stat", None), ("/sys/fs/cgroup/cpu/cpu.stat", None)):
        try:
            with open(stat) as f:
                kv = dict(line.split() for line in f if len(line.split()) == 2)
        except OSError:
            continue
        out["nr_throttled"] = int(kv.get("nr_throttled", 0))
        if "throttled_usec" in kv:
            out["throttled_ms"] = int(kv["throttled_usec"]) / 1e3
        elif "throttled_time" in kv:  # v1: nanoseconds
            out["throttled_ms"] = int(kv["throttled_time"]) / 1e6
        try:
            if quota:
                with open(quota) as f:
                    out["quota"] = f.read().strip()
            else:
                base = os.path.dirname(stat)
                with open(os.path.join(base, "cpu.cfs_quota_us")) as f, \
                        open(os.path.join(base, "cpu.cfs_period_us")) as g:
                    out["quota"] = f"{f.read().strip()} {g.read().strip()}"
        except OSError:
            pass
        break
    return out


def host_cpu_delta(a: dict, b: dict, steps: int) -> dict:
    """what a host-timed loop of `steps` steps cost on the host, from two host_cpu_state() reads"""
    out = {"process_cpu_ms_per_step": round((b["process_cpu_s"] - a["process_cpu_s"]) * 1e3 / steps, 3),
           "cpus_busy": round((b["process_cpu_s"] - a["process_cpu_s"]) / max(1e-9, b["wall_s"] - a["wall_s"]), 2),
           "cpus_usable": len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()}
    if "steal_ms" in a and "steal_ms" in b:
        out["steal_ms_all_cpus"] = round(b["steal_ms"] - a["steal_ms"], 1)
    if "nr_throttled" in a and "nr_throttled" in b:
        out["cgroup_quota"] = b.get("quota")
        out["cgroup_throttled_periods"] = b["nr_throttled"] - a["nr_throttled"]
        if "throttled_ms" in a:
            out["cgroup_throttled_ms"] = round(b["throttled_ms"] - a["throttled_ms"], 3)
    return out


def modmul_count(n: int) -> tuple:
    """Pinned algorithmic work: M(n) = min_c ceil(256/c) (6n + 16 2^c) + 2048 + 16 ceil(256/c)."""
    best = None
    for c in range(4, 23):
        w = -(-256 // c)
        m = w * (6 * n + 16 * 2**c) + 2048 + 16 * w
        if best is None or m < best[0]:
            best = (m, c)
    return best


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def wait_ready(self, timeout: float = 10.0) -> None:
        """block until nvidia-smi has printed its first sample (it takes a while to start)"""
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.01)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float = None, t1: float = None) -> dict:
        """samples read within [t0, t1 + one interval] (the timed region), or the
        first sample after t0 when the region is shorter than the interval"""
        lines = self.lines
        note = "samples within the timed region"
        if t0 is not None:
            inside = [ln for ts, ln in lines if t0 <= ts <= t1 + 0.05]
            if not inside:
                inside = [ln for ts, ln in lines if ts >= t0][:1]
                note = "the first sample after the timed region began (region shorter than the 50 ms interval)"
            lines = inside
        else:
            lines = [ln for _, ln in lines]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "note": note}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "note": note}


def make_inputs(hs, ctx, torch, n: int, device: str):
    """Per curve: device scalars (n*32), device affine bases (n*64, SWU on the GPU),
    plus host copies for the e2e path (scalars + the reference's Jacobian records)."""
    from helioselene_gb300.workload import make_workload
    data = {}
    for curve in (hs.HELIOS, hs.SELENE):
        w = make_workload(curve, n, SEED + curve, edge_fraction=0.01)
        d_u = torch.from_numpy(w.u.reshape(-1).copy()).to(device)
        d_pts = torch.empty(n * 64, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), n, d_pts.data_ptr())
        d_sc = torch.from_numpy(w.scalars.reshape(-1).copy()).to(device)
        torch.cuda.synchronize()
        # host side for the reference-facing path: pinned buffers
        h_sc = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
        h_sc.numpy()[:] = w.scalars.reshape(-1)
        aff = d_pts.cpu().numpy()
        h_jac = torch.empty(n * 120, dtype=torch.uint8, pin_memory=True)
        h_jac.numpy()[:] = affine_to_jac51_fast(aff, n)
        data[curve] = {"w": w, "d_sc": d_sc, "d_pts": d_pts, "h_sc": h_sc, "h_jac": h_jac}
    return data


def affine_to_jac51_fast(aff: np.ndarray, n: int) -> np.ndarray:
    """Vectorised repack of canonical affine (x||y) into helios_jacobian records with Z = 1."""
    words = np.ascontiguousarray(aff.reshape(n, 64)).view(np.uint64).reshape(n, 8)
    out = np.zeros((n, 15), np.uint64)
    m51 = np.uint64((1 << 51) - 1)
    for k, off in ((0, 0), (1, 4)):
        w0, w1, w2, w3 = (words[:, off + i] for i in range(4))
        base = 5 * k
        out[:, base + 0] = w0 & m51
        out[:, base + 1] = ((w0 >> np.uint64(51)) | (w1 << np.uint64(13))) & m51
        out[:, base + 2] = ((w1 >> np.uint64(38)) | (w2 << np.uint64(26))) & m51
        out[:, base + 3] = ((w2 >> np.uint64(25)) | (w3 << np.uint64(39))) & m51
        out[:, base + 4] = (w3 >> np.uint64(12)) & m51
    ident = ~words.any(axis=1)
    out[:, 10] = 1
    out[ident, 0] = 1
    out[ident, 1:5] = 0
    out[ident, 5] = 1
    out[ident, 6:10] = 0
    out[ident, 10] = 0
    return out.view(np.uint8).reshape(-1)


def run_batched(hs, torch, device: str, local: int, steps: int, with_oracle: bool = True) -> dict:
    """Config 3: 1024 independent MSMs, sizes log-uniform in [64, 65536], curve
    Bernoulli(0.5), as one batched launch sequence per curve (two contexts, so the
    two curve groups overlap) against the plain per-call path on the same MSMs."""
    from helioselene_gb300 import autotune
    from helioselene_gb300.workload import batched_stream
    bs = batched_stream(SEED + 3)
    count = 1024
    sizes, curves = bs["sizes"], bs["curves"]
    ctxs = [hs.Context(local), hs.Context(local)]
    t0 = time.time()
    tuned = autotune.load_or_tune(ctxs[0], cache=Path.home() / ".cache" / "helioselene_gb300_autotune.json",
                                  n_max=65536, points_per_class=1 << 20, reps=2)
    for c, name in ((hs.HELIOS, "helios"), (hs.SELENE, "selene")):
        autotune.apply(ctxs[1], c, tuned[name])
    tune_s = time.time() - t0
    groups = {}
    for curve in (hs.HELIOS, hs.SELENE):
        g0 = bs[curve]
        sz = g0["sizes"]
        total = sum(sz)
        d_u = torch.from_numpy(g0["u"].reshape(-1)).to(device)
        d_pts = torch.empty(total * 64, dtype=torch.uint8, device=device)
        d_sc = torch.from_numpy(g0["scalars"].reshape(-1)).to(device)
        d_out = torch.empty(len(sz) * 120, dtype=torch.uint8, device=device)
        d_out_plain = torch.empty(len(sz) * 120, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        ctxs[0].map_to_curve_device(curve, d_u.data_ptr(), total, d_pts.data_ptr())
        torch.cuda.synchronize()
        offs = np.concatenate([[0], np.cumsum(sz)])
        groups[curve] = {"idx": g0["idx"], "sizes": sz, "offs": offs, "d_sc": d_sc, "d_pts": d_pts, "d_out": d_out,
                         "d_out_plain": d_out_plain, "scalars": g0["scalars"]}
    streams = [torch.cuda.ExternalStream(c.stream, device=device) for c in ctxs]

    def batched_once():
        start = torch.cuda.Event(enable_timing=True)
        ends = [torch.cuda.Event(enable_timing=True) for _ in streams]
        start.record(streams[0])
        streams[1].wait_event(start)
        for k, curve in enumerate((hs.HELIOS, hs.SELENE)):
            g = groups[curve]
            ctxs[k].msm_batch_device(curve, g["sizes"], g["d_sc"].data_ptr(), g["d_pts"].data_ptr(),
                                     g["d_out"].data_ptr(), hs.FMT_JACOBIAN51)
            ends[k].record(streams[k])
        for s in streams:
            s.synchronize()
        return max(start.elapsed_time(e) for e in ends)

    batched_once()  # capture the graphs
    times = [batched_once() for _ in range(max(3, steps))]
    batched_ms = statistics.median(times)
    # plain per-call path, the MSMs in stream order on one context, direct launches
    plain_ctx = ctxs[0]
    plain_ctx.set_graphs(False)
    order = np.argsort(np.concatenate([groups[0]["idx"], groups[1]["idx"]]), kind="stable")
    seq = [(0, j) for j in range(len(groups[0]["idx"]))] + [(1, j) for j in range(len(groups[1]["idx"]))]
    seq = [seq[i] for i in order]

    def plain_once():
        s = streams[0]
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for curve, j in seq:
            g = groups[curve]
            o = int(g["offs"][j])
            plain_ctx.msm_device(curve, g["d_sc"].data_ptr() + 32 * o, g["d_pts"].data_ptr() + 64 * o,
                                 g["sizes"][j], g["d_out_plain"].data_ptr() + 120 * j, hs.FMT_JACOBIAN51)
        e.record(s)
        s.synchronize()
        return a.elapsed_time(e)

    plain_once()
    plain_ms = min(plain_once() for _ in range(2))
    plain_ctx.set_graphs(True)
    # same points? compare the serialized 32-byte encodings (Jacobian Z depends on summation order)
    same = True
    for c in (0, 1):
        a = plain_ctx.compress(c, groups[c]["d_out"].cpu().numpy(), hs.FMT_JACOBIAN51)
        p = plain_ctx.compress(c, groups[c]["d_out_plain"].cpu().numpy(), hs.FMT_JACOBIAN51)
        same = same and bool((a == p).all())
    # every batched result against the oracle (one MSM per host thread)
    oracle_ok, oracle_s = None, None
    if with_oracle:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        t1 = time.perf_counter()
        oracle_ok = True
        for c in (0, 1):
            g = groups[c]
            got = plain_ctx.compress(c, g["d_out"].cpu().numpy(), hs.FMT_JACOBIAN51).reshape(-1, 32)
            want = oracle.msm_many(c, g["scalars"], g["d_pts"].cpu().numpy(), g["sizes"])
            oracle_ok = oracle_ok and all(got[i].tobytes() == want[i] for i in range(len(want)))
        oracle_s = time.perf_counter() - t1
    total_pts = int(sizes.sum())
    res = {"msms": count, "points": total_pts, "sizes": "log-uniform [64, 65536], seed-fixed",
           "curves": {"helios": int((curves == 0).sum()), "selene": int((curves == 1).sum())},
           "msms_per_s": count / (batched_ms * 1e-3), "ms": batched_ms,
           "plain_msms_per_s": count / (plain_ms * 1e-3), "plain_ms": plain_ms,
           "speedup_vs_plain": plain_ms / batched_ms, "points_per_s": total_pts / (batched_ms * 1e-3),
           "bit_exact_vs_plain": bool(same), "bit_exact_vs_oracle": oracle_ok,
           "oracle_check": "all 1024 MSMs, one per host thread" if with_oracle else None, "oracle_s": oracle_s,
           "autotune": {"seconds": round(tune_s, 2), **tuned},
           "graph": "one captured launch sequence per curve group, replayed"}
    for c in ctxs:
        c.close()
    return res


def run_serving(hs, torch, device: str, local: int, requests_per_rate: int = 1000, with_oracle: bool = True) -> dict:
    """Config 4: Poisson arrivals of MSM requests, sizes from the mixture 70%
    log-uniform [256, 4096], 25% [4096, 65536], 5% 2^18, curves alternating;
    75% of each request's bases come from a 2^18-point resident pool per curve,
    25% are fresh points sent with the request.  Continuous batching (8 slots,
    batches of up to 2^23 points)
    against the plain path: the same requests one MSM per launch sequence, one
    at a time (a server with one slot and one request per batch, the pooled
    bases gathered as variable bases, as a per-call MSM would take them).  The
    batching server also keeps each pool as a table of window multiples, which
    requests with pooled bases only run over: a second stream of such requests
    (same sizes, no fresh bases) is timed on it, on a server without tables
    (window 0) and on the plain arm."""
    from helioselene_gb300.workload import ORDER, random_field_bytes, random_scalars, serving_sizes
    rng = np.random.default_rng(SEED + 4)
    pool_n = 1 << 18
    res_n = 1 << 19
    pools, fresh, scal = {}, {}, {}
    ctx = hs.Context(local)
    for curve in (hs.HELIOS, hs.SELENE):
        d_u = torch.from_numpy(random_field_bytes(rng, pool_n + res_n).reshape(-1)).to(device)
        d_p = torch.empty((pool_n + res_n) * 64, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), pool_n + res_n, d_p.data_ptr())
        torch.cuda.synchronize()
        allp = d_p.cpu().numpy().reshape(-1, 64)
        pools[curve] = np.ascontiguousarray(allp[:pool_n])
        f = torch.empty(res_n * 64, dtype=torch.uint8, pin_memory=True)
        f.numpy()[:] = allp[pool_n:].reshape(-1)
        fresh[curve] = f
        s = torch.empty(res_n * 2 * 32, dtype=torch.uint8, pin_memory=True)
        s.numpy()[:] = random_scalars(rng, 2 * res_n, ORDER[curve]).reshape(-1)
        scal[curve] = s
    ctx.close()
    perm = torch.empty(2 * res_n * 4, dtype=torch.uint8, pin_memory=True)
    perm.numpy().view(np.uint32)[:] = rng.integers(0, pool_n, 2 * res_n).astype(np.uint32)

    def draw(count, pool_share=0.75):
        n = serving_sizes(rng, count)
        reqs = []
        for i in range(count):
            curve = i % 2
            k = int(n[i])
            npool = int(k * pool_share)
            nfresh = k - npool
            so = int(rng.integers(0, 2 * res_n - k))
            fo = int(rng.integers(0, res_n - nfresh + 1))
            io = int(rng.integers(0, 2 * res_n - npool))
            reqs.append((curve, so, k, io, npool, fo, nfresh))
        return reqs

    def views(r):
        curve, so, k, io, npool, fo, nfresh = r
        sc = scal[curve].numpy()[32 * so:32 * (so + k)]
        idx = perm.numpy().view(np.uint32)[io:io + npool]
        fr = fresh[curve].numpy()[64 * fo:64 * (fo + nfresh)]
        return curve, sc, idx, fr

    def run(srv, reqs, rate, arrivals=None, results=None):
        """submit reqs at the given arrival times (Poisson at `rate`, or all at once)"""
        if arrivals is None:
            arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs))) if rate else np.zeros(len(reqs))
        tickets = []
        with no_python_gc():
            t0 = time.perf_counter()
            for r, at in zip(reqs, arrivals):
                delay = at - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                curve, sc, idx, fr = views(r)
                tickets.append(srv.submit(curve, sc, idx, fr))
            done = [srv.wait(t, 600000) for t in tickets]
            wall = time.perf_counter() - t0
        lat = [d[1] for d in done]
        if results is not None:
            results.extend(d[0] for d in done)
        return {"rate_offered": rate or "all-at-once", "requests": len(reqs), "msms_per_s": len(reqs) / wall,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_points": float(np.mean([r[2] for r in reqs]))}

    out = {"requests_per_rate": requests_per_rate, "pool_points_per_curve": pool_n,
           "mix": "70% [256,4096], 25% [4096,65536], 5% 2^18 log-uniform; 75% pool bases, 25% fresh",
           "plain": "the same requests at the same arrival times, one MSM per launch sequence, one at a time",
           "rates": []}
    srv = hs.Server(local, slots=8, max_batch_points=1 << 23, max_batch_msms=1024)
    gathered = hs.Server(local, slots=8, max_batch_points=1 << 23, max_batch_msms=1024)  # no pool tables
    plain = hs.Server(local, slots=1, max_batch_msms=1)
    for s in (srv, gathered, plain):
        for c in (hs.HELIOS, hs.SELENE):
            if s is not srv:
                s.set_pool_window(c, 0)
            s.set_pool(c, pools[c])
    warm = draw(64)
    run(srv, warm, 0)
    run(plain, warm[:16], 0)
    warm = draw(64, pool_share=1.0)
    run(srv, warm, 0)
    run(gathered, warm, 0)
    run(plain, warm[:16], 0)
    checked = None
    for rate in (1000, 3000, 9000, 0):
        reqs = draw(requests_per_rate)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs))) if rate else np.zeros(len(reqs))
        res_srv, res_plain = [], []
        a = run(srv, reqs, rate, arrivals, res_srv)
        bsec = run(plain, reqs, rate, arrivals, res_plain)
        a["same_as_plain"] = res_srv == res_plain
        out["rates"].append({"serving": a, "plain": bsec})
        if rate == 0:
            checked = (reqs, res_srv)
    # requests with pooled bases only: over the pool tables, gathered, plain
    out["pool_only"] = {"mix": "the same size mixture, every base from the pool", "table_window": 12, "rates": []}
    for rate in (9000, 0):
        reqs = draw(requests_per_rate, pool_share=1.0)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs))) if rate else np.zeros(len(reqs))
        res_t, res_g, res_p = [], [], []
        t = run(srv, reqs, rate, arrivals, res_t)
        g = run(gathered, reqs, rate, arrivals, res_g)
        pl = run(plain, reqs, rate, arrivals, res_p)
        t["same_as_plain"] = res_t == res_p
        g["same_as_plain"] = res_g == res_p
        out["pool_only"]["rates"].append({"table": t, "gathered": g, "plain": pl})
        if rate == 0 and with_oracle:
            sys.path.insert(0, str(ROOT / "oracle"))
            import oracle
            sample = list(range(0, len(reqs), max(1, len(reqs) // 32)))
            ok = True
            for curve in (hs.HELIOS, hs.SELENE):
                sel = [i for i in sample if reqs[i][0] == curve]
                sc = np.concatenate([views(reqs[i])[1].reshape(-1, 32) for i in sel])
                pts = np.concatenate([pools[curve][views(reqs[i])[2]] for i in sel])
                want = oracle.msm_many(curve, sc, pts, [reqs[i][2] for i in sel])
                ok = ok and all(res_t[i] == want[j] for j, i in enumerate(sel))
            out["pool_only"]["bit_exact_vs_oracle"] = ok
            out["pool_only"]["oracle_check"] = f"{len(sample)} of the {len(reqs)} all-at-once requests"
    # a sample of the all-at-once requests against the oracle (pooled + fresh bases)
    if with_oracle and checked:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        reqs, res = checked
        sample = list(range(0, len(reqs), max(1, len(reqs) // 64)))
        ok = True
        t1 = time.perf_counter()
        for curve in (hs.HELIOS, hs.SELENE):
            sel = [i for i in sample if reqs[i][0] == curve]
            sc = np.concatenate([views(reqs[i])[1].reshape(-1, 32) for i in sel])
            pts = np.concatenate([np.concatenate([pools[curve][views(reqs[i])[2]], views(reqs[i])[3].reshape(-1, 64)])
                                  for i in sel])
            want = oracle.msm_many(curve, sc, pts, [reqs[i][2] for i in sel])
            ok = ok and all(res[i] == want[j] for j, i in enumerate(sel))
        out["bit_exact_vs_oracle"] = ok
        out["oracle_check"] = f"{len(sample)} of the {len(reqs)} all-at-once requests, every curve"
        out["oracle_s"] = time.perf_counter() - t1
    out["server_stats"] = srv.stats()
    peak = out["rates"][-1]
    out["msms_per_s"] = peak["serving"]["msms_per_s"]
    out["plain_msms_per_s"] = peak["plain"]["msms_per_s"]
    out["speedup_vs_plain"] = out["msms_per_s"] / out["plain_msms_per_s"]
    srv.close()
    gathered.close()
    plain.close()
    return out


def run_fixed(hs, torch, device: str, local: int, count: int = 4096, chunk: int = 256,
              with_oracle: bool = True, ba_rounds=None) -> dict:
    """Config 5: Pedersen-style commitments r*H + sum v_i G_i over n = 2^20 resident
    generators per curve with device window tables; 4096 commitments per curve,
    submitted 256 at a time from two device scalar buffers used alternately;
    scalars uniform mod order (< 2^255, bit 255 cleared) with 10% of each chunk's
    commitments sparse (one 16-bit value per scalar, <= 16 set bits); all outputs
    normalised to affine with one shared inversion per 16 commitments.  Against
    the plain per-call MSM of n + 1 terms."""
    from helioselene_gb300.workload import random_field_bytes
    n = 1 << 20
    rng = np.random.default_rng(SEED + 5)
    gen = torch.Generator(device=device)
    gen.manual_seed(SEED + 5)
    ctx = hs.Context(local)
    if ba_rounds is not None:
        for curve in (hs.HELIOS, hs.SELENE):
            ctx.set_batch_affine(ba_rounds[curve], 1 << 21, curve)
    stream = torch.cuda.ExternalStream(ctx.stream, device=device)
    nsparse = max(1, chunk // 10)
    out = {"generators": n, "commitments": count, "chunk": chunk, "sparse_fraction": nsparse / chunk}

    def make_scalars():
        sc = torch.randint(0, 256, (chunk, n + 1, 32), dtype=torch.uint8, device=device, generator=gen)
        sc[:, :, 31] &= 0x7F
        sp = sc[:nsparse]
        sp.zero_()
        v16 = torch.randint(0, 65536, (nsparse, n + 1), device=device, generator=gen)
        off = torch.randint(0, 30, (nsparse, n + 1), device=device, generator=gen)
        sp.scatter_(2, off.unsqueeze(2), (v16 & 0xFF).to(torch.uint8).unsqueeze(2))
        sp.scatter_(2, (off + 1).unsqueeze(2), (v16 >> 8).to(torch.uint8).unsqueeze(2))
        return sc

    for curve, name in ((hs.HELIOS, "helios"), (hs.SELENE, "selene")):
        d_u = torch.from_numpy(random_field_bytes(rng, n + 1).reshape(-1)).to(device)
        d_pts = torch.empty((n + 1) * 64, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), n + 1, d_pts.data_ptr())
        torch.cuda.synchronize()
        gens = d_pts.cpu().numpy().reshape(n + 1, 64)
        t0 = time.perf_counter()
        fb = hs.FixedBase(ctx, curve, gens[:n], H=gens[n])
        table_s = time.perf_counter() - t0
        bufs = [make_scalars(), make_scalars()]
        d_out = torch.empty(count * 64, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        fb.commit_device(bufs[0].data_ptr(), chunk, d_out.data_ptr(), hs.FMT_AFFINE)  # warm-up / graph capture
        fb.commit_device(bufs[1].data_ptr(), chunk, d_out.data_ptr(), hs.FMT_AFFINE)
        stream.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for j in range(count // chunk):
            fb.commit_device(bufs[j & 1].data_ptr(), chunk, d_out.data_ptr() + 64 * chunk * j, hs.FMT_AFFINE)
        e.record(stream)
        stream.synchronize()
        fixed_ms = a.elapsed_time(e)
        # plain path: one MSM of n + 1 terms per commitment, on the same device data
        k = 3
        d_plain = torch.empty(k * 120, dtype=torch.uint8, device=device)
        ctx.msm_device(curve, bufs[0][nsparse].data_ptr(), d_pts.data_ptr(), n + 1, d_plain.data_ptr())
        stream.synchronize()
        a.record(stream)
        for j in range(k):
            ctx.msm_device(curve, bufs[0][nsparse + j].data_ptr(), d_pts.data_ptr(), n + 1,
                           d_plain.data_ptr() + 120 * j)
        e.record(stream)
        stream.synchronize()
        plain_ms = a.elapsed_time(e) / k
        aff = d_out.cpu().numpy().reshape(count, 64)
        # the last chunk used buffer (count // chunk - 1) & 1; compare chunk 0 (buffer 0) with the plain path
        got = ctx.compress(curve, aff[nsparse:nsparse + k], hs.FMT_AFFINE)
        want = ctx.compress(curve, d_plain.cpu().numpy(), hs.FMT_JACOBIAN51)
        # a sparse and a dense commitment of chunk 0 against the oracle (blinding
        # last in each commitment's scalars, H appended as generator n)
        oracle_ok = None
        if with_oracle:
            sys.path.insert(0, str(ROOT / "oracle"))
            import oracle
            all_aff = ctx.compress(curve, aff[:chunk], hs.FMT_AFFINE).reshape(chunk, 32)
            oracle_ok = all(oracle.msm_mt(curve, bufs[0][j].cpu().numpy(), gens, oracle.default_threads()) ==
                            all_aff[j].tobytes() for j in (0, nsparse))
        out[name] = {"window": fb.window, "table_bytes": fb.table_bytes, "table_build_s": table_s,
                     "bit_exact_vs_oracle": oracle_ok, "oracle_check": "commitments 0 (sparse) and "
                                                                        f"{nsparse} (dense) of the first chunk",
                     "commitments_per_s": count / (fixed_ms * 1e-3), "ms": fixed_ms,
                     "plain_ms_per_commitment": plain_ms,
                     "speedup_vs_plain": plain_ms * count / fixed_ms,
                     "bit_exact_vs_plain": bool((got == want).all())}
        fb.close()
        del bufs, d_out, d_pts, d_u
        torch.cuda.empty_cache()
    ctx.close()
    return out


def run_sweep(hs, torch, device: str, local: int, flush, with_oracle: bool = True) -> dict:
    """Config 2: single MSMs at n = 2^10, 2^12, ..., 2^22 on both curves, uniform
    scalars mod order, SWU bases, 1% edge slices (zero, order-1, repeated base,
    top-window-only); one MSM at a time, L2 flushed before each, median of 3."""
    from helioselene_gb300.workload import make_workload
    if with_oracle:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
    ctx = hs.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=device)
    out = {}
    for curve, name in ((hs.HELIOS, "helios"), (hs.SELENE, "selene")):
        rows = []
        for lg in range(10, 23, 2):
            n = 1 << lg
            w = make_workload(curve, n, SEED + 2 + lg, edge_fraction=0.01)
            d_u = torch.from_numpy(w.u.reshape(-1).copy()).to(device)
            d_sc = torch.from_numpy(w.scalars.reshape(-1).copy()).to(device)
            d_pts = torch.empty(n * 64, dtype=torch.uint8, device=device)
            d_out = torch.empty(128, dtype=torch.uint8, device=device)
            torch.cuda.synchronize()
            ctx.map_to_curve_device(curve, d_u.data_ptr(), n, d_pts.data_ptr())
            ctx.msm_device(curve, d_sc.data_ptr(), d_pts.data_ptr(), n, d_out.data_ptr())
            torch.cuda.synchronize()
            ts = []
            for _ in range(3):
                with torch.cuda.stream(stream):
                    flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.msm_device(curve, d_sc.data_ptr(), d_pts.data_ptr(), n, d_out.data_ptr())
                b.record(stream)
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b))
            ms = sorted(ts)[1]
            row = {"n": n, "ms": ms, "points_per_s": n / (ms * 1e-3)}
            if with_oracle:
                got = ctx.compress(curve, d_out[:120].cpu().numpy(), hs.FMT_JACOBIAN51).tobytes()
                row["bit_exact_vs_oracle"] = got == oracle.msm_mt(curve, w.scalars, d_pts.cpu().numpy(),
                                                                  oracle.default_threads())
            rows.append(row)
            del d_u, d_sc, d_pts
        out[name] = rows
    ctx.close()
    torch.cuda.empty_cache()
    return out


def run_tree(hs, torch, device: str, local: int, nodes: int = 8192) -> dict:
    """FCMP++ tree-hash layers (src/benchmark_fcmpp.cpp:137-198): a node hash is an
    MSM over the layer's fixed generators followed by to_affine.  A layer of
    `nodes` hashes runs as fixed-base commitments over resident tables with
    affine outputs, against the per-call path (hs_msm_device + affine output) on a
    sample of the same nodes."""
    from helioselene_gb300.workload import ORDER, random_field_bytes, random_scalars
    rng = np.random.default_rng(SEED + 7)
    ctx = hs.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=device)
    out = {"nodes_per_layer": nodes}
    for curve, n, name in ((hs.SELENE, 228, "selene_tree_hash(228)"), (hs.SELENE, 38, "selene_tree_hash(38)"),
                           (hs.HELIOS, 18, "helios_tree_hash(18)")):
        d_u = torch.from_numpy(random_field_bytes(rng, n).reshape(-1)).to(device)
        d_g = torch.empty(n * 64, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), n, d_g.data_ptr())
        torch.cuda.synchronize()
        fb = hs.FixedBase(ctx, curve, d_g.cpu().numpy())
        sc = torch.from_numpy(random_scalars(rng, nodes * n, ORDER[curve]).reshape(-1)).to(device)
        d_out = torch.empty(nodes * 64, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        fb.commit_device(sc.data_ptr(), nodes, d_out.data_ptr(), hs.FMT_AFFINE)
        stream.synchronize()
        ts = []
        for _ in range(3):
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fb.commit_device(sc.data_ptr(), nodes, d_out.data_ptr(), hs.FMT_AFFINE)
            e.record(stream)
            stream.synchronize()
            ts.append(a.elapsed_time(e))
        ms = sorted(ts)[1]
        k = 64
        d_plain = torch.empty(k * 64, dtype=torch.uint8, device=device)
        ctx.msm_device(curve, sc.data_ptr(), d_g.data_ptr(), n, d_plain.data_ptr(), hs.FMT_AFFINE)
        stream.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for j in range(k):
            ctx.msm_device(curve, sc.data_ptr() + 32 * n * j, d_g.data_ptr(), n, d_plain.data_ptr() + 64 * j,
                           hs.FMT_AFFINE)
        e.record(stream)
        stream.synchronize()
        plain_ms = a.elapsed_time(e) / k
        exact = bool(torch.equal(d_out[:k * 64], d_plain))
        out[name] = {"generators": n, "layer_ms": ms, "hashes_per_s": nodes / (ms * 1e-3),
                     "per_call_ms": plain_ms, "speedup_vs_per_call": plain_ms * nodes / ms,
                     "bit_exact_vs_per_call": exact, "window": fb.window}
        fb.close()
    ctx.close()
    return out


def run_verify(hs, torch, device: str, local: int, with_cpu: bool, batch_count: int = 256) -> dict:
    """FCMP++ verification (src/benchmark_fcmpp.cpp:350-439): a batch of proofs
    verifies with one Selene MSM of 522 + 80*batch terms and one Helios MSM of
    265 + 80*batch terms.  Per batch size:
      - the pair of calls from host buffers of reference records (hs_msm, the
        helios_msm_vartime / selene_msm_vartime signature), one after the other
        as the reference benchmark calls them, results read back;
      - the pair on the device, the two MSMs overlapping on two contexts;
      - `batch_count` independent verifications as one batched launch sequence
        per curve (hs_msm_batch_device);
      - the oracle on one host core for one pair (the reference's algorithm)."""
    from helioselene_gb300.workload import ORDER, random_field_bytes, random_scalars
    rng = np.random.default_rng(SEED + 11)
    H, S = hs.HELIOS, hs.SELENE
    ctxs = {H: hs.Context(local), S: hs.Context(local)}
    ctxs[S].set_priority(True)
    streams = {c: torch.cuda.ExternalStream(x.stream, device=device) for c, x in ctxs.items()}
    V = batch_count
    out = {"batched_verifications": V}
    if with_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle

    def pair_timed(launch):
        start = torch.cuda.Event(enable_timing=True)
        ends = {c: torch.cuda.Event(enable_timing=True) for c in streams}
        start.record(streams[H])
        streams[S].wait_event(start)
        for c in (S, H):
            launch(c)
            ends[c].record(streams[c])
        for st in streams.values():
            st.synchronize()
        return max(start.elapsed_time(e) for e in ends.values())

    for batch in (1, 2, 4, 10):
        sizes = {S: 522 + 80 * batch, H: 265 + 80 * batch}
        g = {}
        for c, n in sizes.items():
            d_u = torch.from_numpy(random_field_bytes(rng, n * V).reshape(-1)).to(device)
            d_pts = torch.empty(n * V * 64, dtype=torch.uint8, device=device)
            torch.cuda.synchronize()
            ctxs[c].map_to_curve_device(c, d_u.data_ptr(), n * V, d_pts.data_ptr())
            d_sc = torch.from_numpy(random_scalars(rng, n * V, ORDER[c]).reshape(-1)).to(device)
            torch.cuda.synchronize()
            aff = d_pts[:n * 64].cpu().numpy()
            g[c] = {"n": n, "d_sc": d_sc, "d_pts": d_pts, "h_sc": d_sc[:n * 32].cpu().numpy(), "aff": aff,
                    "h_jac": affine_to_jac51_fast(aff, n),
                    "d_out": torch.empty(V * 120, dtype=torch.uint8, device=device)}

        def host_pair():
            return [ctxs[c].msm(c, g[c]["h_sc"], g[c]["h_jac"], hs.FMT_JACOBIAN51, hs.FMT_JACOBIAN51) for c in (S, H)]

        for _ in range(3):
            got = host_pair()
        ts = []
        for _ in range(20):
            t0 = time.perf_counter()
            host_pair()
            ts.append(time.perf_counter() - t0)
        host_ms = statistics.median(ts) * 1e3

        def dev(c):
            ctxs[c].msm_device(c, g[c]["d_sc"].data_ptr(), g[c]["d_pts"].data_ptr(), g[c]["n"],
                               g[c]["d_out"].data_ptr(), hs.FMT_JACOBIAN51)

        for _ in range(3):
            pair_timed(dev)
        dev_ms = statistics.median([pair_timed(dev) for _ in range(20)])

        def bat(c):
            ctxs[c].msm_batch_device(c, [g[c]["n"]] * V, g[c]["d_sc"].data_ptr(), g[c]["d_pts"].data_ptr(),
                                     g[c]["d_out"].data_ptr(), hs.FMT_JACOBIAN51)

        pair_timed(bat)  # capture the graphs
        bat_ms = statistics.median([pair_timed(bat) for _ in range(5)])
        # the batched results' first verification against the per-call pair
        exact = all((ctxs[c].compress(c, g[c]["d_out"][:120].cpu().numpy(), hs.FMT_JACOBIAN51) ==
                     ctxs[c].compress(c, np.frombuffer(got[k], np.uint8), hs.FMT_JACOBIAN51)).all()
                    for k, c in enumerate((S, H)))
        row = {"selene_n": sizes[S], "helios_n": sizes[H], "host_pair_ms": host_ms, "device_pair_ms": dev_ms,
               "batched_ms": bat_ms, "verifications_per_s": V / (bat_ms * 1e-3), "bit_exact_batched_vs_call": exact}
        if with_cpu:
            t0 = time.perf_counter()
            want = [oracle.msm(c, g[c]["h_sc"].reshape(-1, 32), g[c]["aff"].reshape(-1, 64)) for c in (S, H)]
            row["cpu_port_pair_ms_1core"] = (time.perf_counter() - t0) * 1e3
            row["bit_exact_vs_oracle"] = all(ctxs[c].msm(c, g[c]["h_sc"], g[c]["aff"]) == want[k]
                                             for k, c in enumerate((S, H)))
        out[f"batch={batch}"] = row
    for c in ctxs.values():
        c.close()
    return out


def run_scalar_mul(hs, torch, ctxs, data, n: int, flush) -> dict:
    """Independent variable-time scalar multiplications s_i P_i (the n = 1 MSM of
    the serving path, helios_scalarmult_vartime) over the bench's scalars and
    bases, device-resident, one thread per pair."""
    out = {}
    for curve, name in ((hs.HELIOS, "helios"), (hs.SELENE, "selene")):
        c = ctxs[curve]
        s = torch.cuda.ExternalStream(c.stream, device=data[curve]["d_pts"].device)
        d_out = torch.empty(n * 96, dtype=torch.uint8, device=data[curve]["d_pts"].device)
        args = (data[curve]["d_sc"].data_ptr(), data[curve]["d_pts"].data_ptr(), n, d_out.data_ptr())
        c.scalar_mul_device(curve, *args, hs.FMT_AFFINE)
        torch.cuda.synchronize()
        ts = []
        for _ in range(3):
            with torch.cuda.stream(s):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            c.scalar_mul_device(curve, *args, hs.FMT_AFFINE)
            b.record(s)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        ms = sorted(ts)[1]
        out[name] = {"pairs": n, "ms": ms, "scalar_mults_per_s": n / (ms * 1e-3), "out_fmt": "affine"}
    return out


IMAD_PER_MODSQR = {0: 88, 1: 176}  # F_p, F_q squaring: 36 products + the same reduction
# per decoded point: x^3 - 3x + b, one 4-bit-window exponentiation (256 S + 78 M), the root check
DECODE_SQR, DECODE_MUL = 258, 80


def run_decompress(hs, torch, ctxs, data, n: int, flush, imad_peak: float) -> dict:
    """Point decoding on the device (hs_decompress_device) over the bench bases'
    32-byte encodings, and one MSM fed with encodings through hs_msm
    (HS_FMT_COMPRESSED, host buffers, decoding inside the timed call)."""
    out = {}
    for curve, name in ((hs.HELIOS, "helios"), (hs.SELENE, "selene")):
        c = ctxs[curve]
        s = torch.cuda.ExternalStream(c.stream, device=data[curve]["d_pts"].device)
        enc = c.compress(curve, data[curve]["d_pts"].cpu().numpy(), hs.FMT_AFFINE)
        data[curve]["enc"] = enc
        d_in = torch.from_numpy(enc.copy()).to(data[curve]["d_pts"].device)
        d_out = torch.empty(n * 64, dtype=torch.uint8, device=d_in.device)
        d_valid = torch.empty(n, dtype=torch.uint8, device=d_in.device)
        torch.cuda.synchronize()
        ts = []
        for i in range(4):
            with torch.cuda.stream(s):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            c.decompress_device(curve, d_in.data_ptr(), n, d_out.data_ptr(), d_valid.data_ptr())
            b.record(s)
            torch.cuda.synchronize()
            if i:
                ts.append(a.elapsed_time(b))
        ok = bool(torch.equal(d_out, data[curve]["d_pts"]))
        ms = min(ts)
        work = n * (DECODE_SQR * IMAD_PER_MODSQR[curve] + DECODE_MUL * IMAD_PER_MODMUL[curve])
        h_sc = data[curve]["h_sc"].numpy()
        h_enc = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
        h_enc.numpy()[:] = enc
        c.msm(curve, h_sc, h_enc.numpy(), hs.FMT_COMPRESSED, hs.FMT_JACOBIAN51)
        t0 = time.perf_counter()
        for _ in range(3):
            c.msm(curve, h_sc, h_enc.numpy(), hs.FMT_COMPRESSED, hs.FMT_JACOBIAN51)
        e2e = (time.perf_counter() - t0) / 3
        out[name] = {"points": n, "ms": ms, "points_per_s": n / (ms * 1e-3), "round_trip_exact": ok,
                     "roofline": {"bound": "imad", "achieved": work / (ms * 1e-3) / 1e12, "peak": imad_peak / 1e12,
                                  "unit": "T IMAD/s", "frac": work / (ms * 1e-3) / imad_peak if imad_peak else None,
                                  "work": f"{DECODE_SQR} squarings + {DECODE_MUL} products per point, "
                                          "IMAD-eq as for the MSM"},
                     "msm_from_encodings_e2e": {"ms": e2e * 1e3, "points_per_s": n / e2e,
                                                "api": "hs_msm(point_fmt=HS_FMT_COMPRESSED), pinned host buffers, "
                                                       "32 B scalar + 32 B encoding per point"}}
    return out


def executed_per_entry(rounds: int, curve: int) -> float:
    """IMAD-equivalents executed per (point, window) entry by the accumulation with
    `rounds` batch-affine rounds: round r adds 2^-r pairs per entry at 5M + 1S, the
    fold 2^-rounds items per entry at 8M + 2S"""
    m, s = IMAD_PER_MODMUL[curve], IMAD_PER_MODSQR[curve]
    pair, madd = 5 * m + s, 8 * m + 2 * s
    return sum(pair / 2**r for r in range(1, rounds + 1)) + madd / 2**rounds


def _traffic(rounds: int, c: int):
    t = ACC_TRAFFIC.get(rounds)
    return (t["bytes"][c], t["capture"][c]) if t and t["bytes"][c] is not None else (None, None)


def traffic_of(rr) -> float:
    """the captured accumulation-phase DRAM bytes per MSM, mean of the curves (None if not captured)"""
    vals = [_traffic(rr[c], c)[0] for c in (0, 1)]
    return sum(vals) / 2 if None not in vals else None


def traffic_source(rr) -> str:
    parts = []
    for c, name in ((0, "Helios"), (1, "Selene")):
        b, cap = _traffic(rr[c], c)
        parts.append(f"{name}: " + (f"{b / 1e6:.1f} MB, ncu capture {cap}" if b else "no capture of this form"))
    return "; ".join(parts)


def probe_rates(rates: dict, torch, local: int, clk: dict) -> dict:
    """the IMAD probe's instruction rates, per SM per clock at the SM clock seen
    in the timed region (the denominator of every roofline fraction here)"""
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    out = {"sm_count": sms, "sm_mhz": mhz, "unit": "instructions per SM per clock",
           "note": "mad_lo_hi: alternating mad.lo/mad.hi (1 IMAD-eq each); mad_wide: mad.wide.u32 (one 32x32->64 "
                   "product, 2 IMAD-eq); peak = max(mad_lo_hi, 2 x mad_wide) x SMs x clock"}
    for k, v in rates.items():
        out[k] = round(v / (sms * mhz * 1e6), 2) if mhz else None
    return out


def cpu_baseline_leg(data, n: int, gpu_results: dict) -> dict:
    """The oracle port on all host cores, on the same workload; also checks the GPU results."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    threads = oracle.default_threads()
    t0 = time.perf_counter()
    match = True
    for curve, d in data.items():
        pts = d["d_pts"].cpu().numpy()
        r = oracle.msm_mt(curve, d["w"].scalars, pts, threads)
        match = match and (r == gpu_results.get(curve))
    dt = time.perf_counter() - t0
    dec = {}
    for curve, d in data.items():
        if "enc" not in d:
            continue
        k = min(n, 1 << 14)
        t1 = time.perf_counter()
        pts, bad = oracle.decompress(curve, d["enc"][:32 * k])
        dec[curve] = {"points_per_s": k / (time.perf_counter() - t1), "cores": 1, "sample": f"{k} encodings",
                      "matches_gpu_bases": bool(bad == 0 and pts.tobytes() == d["d_pts"][:64 * k].cpu().numpy().tobytes())}
    return {"value": 2 * n / dt, "unit": "points/s", "cores": threads, "kind": "port",
            "decompress": dec,
            "sample": f"the full timed workload (Helios + Selene MSM, n=2^{n.bit_length() - 1} each), split into "
                      f"{threads} per-thread sub-MSMs summed with the group law, one pass",
            "seconds": dt, "bit_exact_vs_gpu": bool(match)}


def run_ours(args) -> None:
    import torch

    import helioselene_gb300 as hs

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    ctx = hs.Context(local)
    ctx2 = hs.Context(local)  # the Selene MSM of a step runs on its own stream, overlapping the Helios one
    # the two curves already overlap on two streams, so the window split is off for
    # the throughput step; the Selene context (the longer MSM) gets the
    # high-priority stream so its blocks are scheduled first and the Helios MSM
    # fills the SMs its tail leaves idle
    head_split = 0 if args.split is None else args.split
    ctx.set_split(head_split)
    ctx2.set_split(head_split)
    if args.priority == "selene":
        ctx2.set_priority(True)
    elif args.priority == "helios":
        ctx.set_priority(True)
    # the accumulation form of each curve (batch-affine rounds): the library's
    # defaults, or set for every kind of plan by --ba-rounds
    rr = list(DEFAULT_BA_ROUNDS)
    rr_host = list(HOST_BA_ROUNDS)
    if args.ba_rounds is not None:
        rr = [int(x) for x in str(args.ba_rounds).split(",")]
        rr = rr * 2 if len(rr) == 1 else rr
        rr_host = list(rr)
        for c in (ctx, ctx2):
            for curve in (hs.HELIOS, hs.SELENE):
                c.set_batch_affine(rr[curve], 1 << 21, curve)
    ctxs = {hs.HELIOS: ctx, hs.SELENE: ctx2}
    n = args.n
    data = make_inputs(hs, ctx, torch, n, device)
    streams = {c: torch.cuda.ExternalStream(x.stream, device=device) for c, x in ctxs.items()}
    stream = streams[hs.HELIOS]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    d_out = torch.empty(2 * 128, dtype=torch.uint8, device=device)
    torch.cuda.synchronize()

    def launch_pair():
        for curve in (hs.HELIOS, hs.SELENE):
            ctxs[curve].msm_device(curve, data[curve]["d_sc"].data_ptr(), data[curve]["d_pts"].data_ptr(), n,
                                   d_out.data_ptr() + 128 * curve, hs.FMT_JACOBIAN51)

    def run_steps(k):
        """k steps issued back to back on the two context streams; events bracket all of them"""
        start, end, end_s = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        start.record(stream)
        streams[hs.SELENE].wait_event(start)
        for _ in range(k):
            launch_pair()
        end_s.record(streams[hs.SELENE])
        stream.wait_event(end_s)
        end.record(stream)
        return start, end

    def isolated_step():
        """one step alone: L2 flushed and the device synchronised before its events"""
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        start, end = run_steps(1)
        torch.cuda.synchronize()
        return start.elapsed_time(end)

    run_steps(args.warmup)
    torch.cuda.synchronize()
    # results as the reference returns them (Jacobian records), serialized for the bit-exact check
    out_host = d_out.cpu().numpy()
    results = {c: ctx.compress(c, out_host[128 * c:128 * c + 120], hs.FMT_JACOBIAN51).tobytes()
               for c in (hs.HELIOS, hs.SELENE)}

    # ---- timed region: device-resident inputs, K steps of both curves ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches + ctx2.launches
    with ClockSampler(local) as clocks:
        clocks.wait_ready()
        w0 = time.time()
        t_start, t_end = run_steps(args.steps)
        torch.cuda.synchronize()
        w1 = time.time()
    launches = ctx.launches + ctx2.launches - launches0
    ms = t_start.elapsed_time(t_end)
    if dist:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = ws * 2 * n / (ms_per_step * 1e-3)
    isolated_ms = sorted(isolated_step() for _ in range(5))[2]

    # per-curve latency, one MSM at a time; then the roofline pass: the unsplit
    # batch path of the same MSM with its accumulation launch timed by events on
    # the context stream (a split MSM runs two accumulations concurrently, which
    # per-launch events cannot separate)
    per_curve = {}
    prof_total = {"ms": 0.0, "work": 0.0, "executed": 0.0, "launches": 0}
    for curve, name in ((hs.HELIOS, "helios"), (hs.SELENE, "selene")):
        c = ctxs[curve]
        s = streams[curve]
        args_dev = (data[curve]["d_sc"].data_ptr(), data[curve]["d_pts"].data_ptr())

        def timed(fn):
            ts = []
            for _ in range(3):
                with torch.cuda.stream(s):
                    flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                fn()
                b.record(s)
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b))
            return min(ts)

        c.set_split(SPLIT_DEFAULT if args.split is None else args.split)  # a lone MSM: the library default
        t_split = timed(lambda: c.msm_device(curve, *args_dev, n, d_out.data_ptr(), hs.FMT_JACOBIAN51))
        c.set_split(head_split)
        c.profile(True)
        c.profile_read(reset=True)
        t_plain = timed(lambda: c.msm_batch_device(curve, [n], *args_dev, d_out.data_ptr(), hs.FMT_JACOBIAN51))
        pr = c.profile_read(reset=True)
        c.profile(False)
        per_curve[name] = {"ms": t_split, "points_per_s": n / (t_split * 1e-3), "unsplit_ms": t_plain,
                           "accumulate_ms": pr["accumulate_ms"] / max(1, pr["accumulate_launches"])}
        prof_total["ms"] += pr["accumulate_ms"]
        prof_total["launches"] += pr["accumulate_launches"]
        prof_total["work"] += pr["entries"] * 6 * IMAD_PER_MODMUL[curve]
        prof_total["executed"] += pr["entries"] * executed_per_entry(rr[curve], curve)

    # ---- e2e: reference-facing call with host buffers ----
    # Each e2e step is one isolated pair of calls (nothing of the next step
    # overlaps its tail), so the contexts use the library's default window split,
    # which shortens a lone MSM's tail.  The heavier Selene call is started first:
    # the device's shared copy stream then delivers its inputs first.
    e2e_split = SPLIT_DEFAULT if args.split is None else args.split
    for c in ctxs.values():
        c.set_split(e2e_split)
    # at least 150 steps (about 0.9 s): stalled steps, seen in about one run in
    # six, cost the mean about the same fraction on average whatever the loop's
    # length, but a longer loop spreads that cost evenly over the runs
    e2e_steps = max(150, args.steps)
    for _ in range(2):
        for curve in (hs.HELIOS, hs.SELENE):
            ctxs[curve].msm(curve, data[curve]["h_sc"].numpy(), data[curve]["h_jac"].numpy(), hs.FMT_JACOBIAN51,
                            hs.FMT_JACOBIAN51)
    if dist:
        dist.barrier()
    # the host link's rate right now, for reading the e2e number: one copy of the
    # Selene records (pinned) to the device
    h2d_probe = torch.empty(data[hs.SELENE]["h_jac"].numel(), dtype=torch.uint8, device=device)
    h2d_gbps = []
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        h2d_probe.copy_(data[hs.SELENE]["h_jac"], non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        h2d_gbps.append(h2d_probe.numel() / (a.elapsed_time(b) * 1e6))
    del h2d_probe
    # the two curves from two host threads of a pool (one context each), as a
    # caller would overlap them
    from concurrent.futures import ThreadPoolExecutor
    args_of = {c: (c, data[c]["h_sc"].numpy(), data[c]["h_jac"].numpy(), hs.FMT_JACOBIAN51, hs.FMT_JACOBIAN51)
               for c in (hs.SELENE, hs.HELIOS)}
    with ThreadPoolExecutor(max_workers=2) as pool:
        # ten warm-up pairs: the device has idled through the host-side work before
        for _ in range(10):
            for f in [pool.submit(ctxs[c].msm, *args_of[c]) for c in (hs.SELENE, hs.HELIOS)]:
                f.result()
        e2e_step_ms, e2e_calls = [], []

        def timed_call(c):
            # the calling thread's CPU time beside its wall time: a thread that was
            # descheduled shows less CPU than wall time, one that waited on the
            # device (the runtime spins in its synchronise) about as much
            t, u = time.perf_counter(), time.thread_time()
            ctxs[c].msm(*args_of[c])
            return t, time.perf_counter(), time.thread_time() - u

        with no_python_gc():
            cpu0 = host_cpu_state()
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                ts = time.perf_counter()
                fut = {c: pool.submit(timed_call, c) for c in (hs.SELENE, hs.HELIOS)}
                span = {c: f.result() for c, f in fut.items()}
                te = time.perf_counter()
                e2e_step_ms.append((te - ts) * 1e3)
                e2e_calls.append({("selene" if c == hs.SELENE else "helios"):
                                  [round((a - ts) * 1e3, 3), round((b - ts) * 1e3, 3), round(u * 1e3, 3)]
                                  for c, (a, b, u) in span.items()})
            e2e_s = (time.perf_counter() - t0) / e2e_steps
            e2e_host = host_cpu_delta(cpu0, host_cpu_state(), e2e_steps)
        e2e_med = statistics.median(e2e_step_ms)
        e2e_slow = [{"step": i, "ms": round(t, 3), "calls_start_end_cpu_ms": e2e_calls[i]}
                    for i, t in enumerate(e2e_step_ms) if t > 1.5 * e2e_med]
        # the same calls from pageable copies of the inputs (ordinary arrays, as
        # a caller of the drop-ins holds them)
        args_pg = {c: (c, np.array(data[c]["h_sc"].numpy()), np.array(data[c]["h_jac"].numpy()), hs.FMT_JACOBIAN51,
                       hs.FMT_JACOBIAN51) for c in (hs.SELENE, hs.HELIOS)}
        for _ in range(3):
            for f in [pool.submit(ctxs[c].msm, *args_pg[c]) for c in (hs.SELENE, hs.HELIOS)]:
                f.result()
        pg_step_ms = []
        with no_python_gc():
            for _ in range(e2e_steps):
                ts = time.perf_counter()
                for f in [pool.submit(ctxs[c].msm, *args_pg[c]) for c in (hs.SELENE, hs.HELIOS)]:
                    f.result()
                pg_step_ms.append((time.perf_counter() - ts) * 1e3)
        del args_pg
    e2e_pageable = {"value": ws * 2 * n / (statistics.mean(pg_step_ms) * 1e-3), "unit": "points/s",
                    "median_step_value": ws * 2 * n / (statistics.median(pg_step_ms) * 1e-3),
                    "steps": e2e_steps, "api": "the same calls with the inputs in pageable host memory (numpy arrays)"}
    for c in ctxs.values():
        c.set_split(head_split)
    # the same pair as one hs_msm_batch call (both curves, one context)
    pair = [(c, data[c]["h_sc"].numpy(), data[c]["h_jac"].numpy()) for c in (hs.SELENE, hs.HELIOS)]
    ctx.msm_batch(pair, hs.FMT_JACOBIAN51, hs.FMT_JACOBIAN51)
    with no_python_gc():
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.msm_batch(pair, hs.FMT_JACOBIAN51, hs.FMT_JACOBIAN51)
        e2e_batch_s = (time.perf_counter() - t0) / e2e_steps
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    # ---- roofline of the dominant kernel (bucket accumulation) ----
    imad_peak = ctx.measure_imad_peak()
    imad_rates = ctx.measure_imad_rates()
    achieved = prof_total["work"] / (prof_total["ms"] * 1e-3) if prof_total["ms"] > 0 else 0.0
    acc_ms = prof_total["ms"] / max(1, prof_total["launches"])
    batched = None
    if not args.no_batched:
        batched = run_batched(hs, torch, device, local, args.steps, with_oracle=not args.no_cpu)
    serving = None
    if not args.no_serving:
        serving = run_serving(hs, torch, device, local, with_oracle=not args.no_cpu)
    fixed = None
    if not args.no_fixed:
        fixed = run_fixed(hs, torch, device, local, with_oracle=not args.no_cpu,
                          ba_rounds=rr if args.ba_rounds is not None else None)
    smul = None
    if not args.no_scalar_mul:
        smul = run_scalar_mul(hs, torch, ctxs, data, n, flush)
    tree = None
    if not args.no_tree:
        tree = run_tree(hs, torch, device, local)
    verify = None
    if not args.no_verify:
        verify = run_verify(hs, torch, device, local, with_cpu=(ws == 1 and not args.no_cpu))
    sweep = None
    if not args.no_sweep:
        sweep = run_sweep(hs, torch, device, local, flush, with_oracle=not args.no_cpu)
    decode = None
    if not args.no_decompress:
        decode = run_decompress(hs, torch, ctxs, data, n, flush, imad_peak)
    m_n, c_star = modmul_count(n)
    whole = m_n * (IMAD_PER_MODMUL[0] + IMAD_PER_MODMUL[1]) / (ms_per_step * 1e-3)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n": n, "curves": ["helios", "selene"], "parallelism": f"replicas{ws}",
                       "window_split_min_points": head_split,
                       "streams": "Helios and Selene MSMs on two context streams" + (
                           f", {args.priority.capitalize()}'s of high priority" if args.priority != "none" else ""),
                       "l2": "inputs of one step (2 x 96 MiB scalars + bases, plus the bucket workspaces) exceed "
                             "L2 (129 MB); steps are issued back to back and the events bracket all K of them",
                       "isolated_ms_per_step": isolated_ms,
                       "isolated_note": "median of 5 single steps, each after a 256 MiB L2 flush and a synchronise",
                       "inputs": "device-resident scalars + canonical affine bases"},
            "per_curve": per_curve,
            "clocks": clocks.summary(w0, w1),
            "gpu_launches": launches,
            "e2e": {"value": ws * 2 * n / e2e_s, "unit": "points/s",
                    "h2d_bytes_per_step": 2 * n * (32 + 120), "d2h_bytes_per_step": 2 * 120,
                    "api": "hs_msm(point_fmt=HS_FMT_JACOBIAN51, out_fmt=HS_FMT_JACOBIAN51), pinned host buffers",
                    "calls": "one per curve from a pool of two host threads, Selene first", "window_split_min": e2e_split,
                    "ba_rounds": {"helios": rr_host[0], "selene": rr_host[1]},
                    "python_gc": "paused during the timed steps (collected and frozen first)",
                    "step_ms": {"median": statistics.median(e2e_step_ms), "min": min(e2e_step_ms),
                                "max": max(e2e_step_ms), "all": [round(t, 3) for t in e2e_step_ms]},
                    "slow_steps": e2e_slow,
                    "host": e2e_host,
                    "pageable": e2e_pageable,
                    "median_step_value": ws * 2 * n / (statistics.median(e2e_step_ms) * 1e-3),
                    "h2d_GBps_before": round(statistics.median(h2d_gbps), 1),
                    "one_batch_call": {"value": ws * 2 * n / e2e_batch_s, "unit": "points/s",
                                       "api": "hs_msm_batch with both MSMs (HS_FMT_JACOBIAN51 in and out)"}},
            "roofline": {"bound": "imad", "achieved": achieved / 1e12, "peak": imad_peak / 1e12,
                         "unit": "T IMAD/s", "frac": achieved / imad_peak if imad_peak else None,
                         "traffic": traffic_of(rr), "traffic_unit": "bytes per MSM's accumulation phase "
                                                                   "(DRAM read + write), mean of the two curves",
                         "traffic_source": traffic_source(rr),
                         "kernel": "bucket accumulation phase: " + ("; ".join(
                             f"{name} " + ("k_accumulate (XYZZ)" if rr[c] == 0 else
                                          f"{rr[c]} batch-affine round(s) (k_ba_pairs, k_ba_invert, k_ba_finish) "
                                          "+ XYZZ fold (k_accumulate_level)")
                             for c, name in ((0, "Helios"), (1, "Selene")))),
                         "ba_rounds": {"helios": rr[0], "selene": rr[1]},
                         "work": "point-window entries x 6 modmul (batch-affine bucket add) x IMAD-eq per modmul "
                                 "(F_p 144, F_q 232), summed over one Helios and one Selene launch",
                         "peak_source": "measured in this run by hs_measure_imad_peak (the faster of mad.lo/mad.hi "
                                        "and mad.wide.u32 chains on every SM)",
                         "accumulate_ms_per_launch": acc_ms,
                         "executed_frac": (prof_total["executed"] / (prof_total["ms"] * 1e-3) / imad_peak
                                           if imad_peak and prof_total["ms"] > 0 else None),
                         "executed_note": "the same launches counted with the products they execute: XYZZ mixed "
                                          "addition 8 products + 2 squares per item; a batch-affine pair 5 "
                                          "products + 1 square (prefix, walk back, lambda, y) plus the shared "
                                          "inversion",
                         "whole_msm_frac": whole / imad_peak if imad_peak else None,
                         "pinned_entries": "n x ceil(256/c) per MSM (c = 16 at n = 2^20: 16 windows), "
                                           "6 modmul each",
                         "probe_rates": probe_rates(imad_rates, torch, local, clocks.summary(w0, w1))},
        }
        if not args.no_batched:
            line["batched"] = batched
        if not args.no_serving:
            line["serving"] = serving
        if not args.no_fixed:
            line["fixed_base"] = fixed
        if not args.no_decompress:
            line["decompress"] = decode
        if not args.no_sweep:
            line["sweep"] = sweep
        if not args.no_tree:
            line["tree_hash"] = tree
        if not args.no_verify:
            line["fcmpp_verify"] = verify
        if not args.no_scalar_mul:
            line["scalar_mul"] = smul
        if ws == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline_leg(data, n, results)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    ctx.close()
    ctx2.close()


def _reference_library():
    """The reference library compiled from the helioselene sources by oracle/Makefile
    (oracle/_ref/libhsref.so), where it exists for this host; else None."""
    import ctypes
    path = ROOT / "oracle" / "_ref" / "libhsref.so"
    if not path.exists():
        return None
    try:
        lib = ctypes.CDLL(str(path))
    except OSError:
        return None
    lib.ref_msm.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.ref_msm.restype = ctypes.c_int
    return lib


def _reference_msm_mt(ref, oracle, curve, scalars, pts, threads):
    """the reference's helios_msm_vartime / selene_msm_vartime on `threads` host
    threads (one slice of the terms each, the call releases the GIL), the partial
    results added with the group law"""
    from concurrent.futures import ThreadPoolExecutor
    import ctypes
    n = scalars.shape[0]
    cuts = np.linspace(0, n, threads + 1).astype(np.int64)

    def part(j):
        lo, hi = int(cuts[j]), int(cuts[j + 1])
        s = np.ascontiguousarray(scalars[lo:hi])
        p = np.ascontiguousarray(pts.reshape(n, 64)[lo:hi])
        out = np.zeros(32, np.uint8)
        assert ref.ref_msm(curve, out.ctypes.data_as(ctypes.c_void_p), s.ctypes.data_as(ctypes.c_void_p),
                           p.ctypes.data_as(ctypes.c_void_p), hi - lo) == 0
        return out

    with ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(part, range(threads)))
    acc = np.zeros(64, np.uint8)
    for enc in parts:
        pt, bad = oracle.decompress(curve, enc)
        acc = np.frombuffer(oracle.point_add(curve, acc, pt if not bad else np.zeros(64, np.uint8)), np.uint8)
    return oracle.compress(curve, acc).tobytes()


def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from helioselene_gb300.workload import make_workload
    n = args.n
    threads = oracle.default_threads()
    ref = _reference_library()
    data = {}
    for curve in (0, 1):
        w = make_workload(curve, n, SEED + curve, edge_fraction=0.01)
        pts = oracle.map_to_curve_mt(curve, w.u.reshape(-1), threads)
        data[curve] = (w.scalars, pts)
    if ref is not None:
        kind = "reference"
        sample = (f"full workload per step, {threads} threads: the reference's helios_msm_vartime / "
                  "selene_msm_vartime (its x64 radix-2^51 code compiled from its sources by oracle/Makefile) on one "
                  "slice of the terms per thread, partial results added with the group law")

        def step(curve):
            return _reference_msm_mt(ref, oracle, curve, data[curve][0], data[curve][1], threads)
    else:
        kind = "port"
        sample = (f"full workload per step, {threads} threads, per-thread sub-MSMs (the reference Pippenger "
                  "restated in C, oracle/hs_oracle.c) summed with the group law; the reference library compiled "
                  "from its sources (oracle/_ref) is absent on this host")

        def step(curve):
            return oracle.msm_mt(curve, data[curve][0], data[curve][1], threads)
    for _ in range(args.warmup):
        for curve in (0, 1):
            step(curve)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for curve in (0, 1):
            step(curve)
    dt = (time.perf_counter() - t0) / args.steps
    value = 2 * n / dt
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "n": n, "curves": ["helios", "selene"]},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched (1024 uneven MSMs) section")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving (Poisson arrivals) section")
    ap.add_argument("--no-fixed", action="store_true", help="skip the fixed-base commitment section")
    ap.add_argument("--no-decompress", action="store_true", help="skip the point-decoding section")
    ap.add_argument("--no-sweep", action="store_true", help="skip the n = 2^10 .. 2^22 single-MSM sweep")
    ap.add_argument("--no-tree", action="store_true", help="skip the FCMP++ tree-hash layer section")
    ap.add_argument("--no-verify", action="store_true", help="skip the FCMP++ verification-batch section")
    ap.add_argument("--no-scalar-mul", action="store_true", help="skip the independent scalar-multiplication section")
    ap.add_argument("--priority", default="selene", choices=["selene", "helios", "none"],
                    help="the curve whose context stream gets the high priority in the throughput step")
    ap.add_argument("--ba-rounds", default=None,
                    help="batch-affine accumulation rounds for plans of >= 2^21 entries, one value for both curves "
                         "or 'helios,selene' (0: XYZZ; default: the library's)")
    ap.add_argument("--split", type=int, default=None,
                    help="window-split threshold in points for single MSMs (0: off; default: the library's)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
