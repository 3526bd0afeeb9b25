"""Run the batched configuration on one GPU and print its time:

    python -m helioselene_gb300.batchrun [reps]

1024 independent MSMs of log-uniform sizes in [64, 65536] on either curve
(``workload.batched_stream``, 9.85M points), one ``hs_msm_batch_device`` call
per curve group on one context, with the built-in window rule.  Two calls
warm up (and capture the launch sequences); ``reps`` calls are timed.  Needs
PyTorch for the device buffers."""

import json
import sys
import time


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    reps = int(argv[0]) if argv else 2
    import torch

    import helioselene_gb300 as hs
    from helioselene_gb300.workload import BENCH_SEED, batched_stream

    bs = batched_stream(BENCH_SEED + 3)
    ctx = hs.Context(0)
    groups = {}
    for curve in (hs.HELIOS, hs.SELENE):
        g = bs[curve]
        total = sum(g["sizes"])
        d_u = torch.from_numpy(g["u"].reshape(-1)).cuda()
        d_pts = torch.empty(total * 64, dtype=torch.uint8, device="cuda")
        d_sc = torch.from_numpy(g["scalars"].reshape(-1)).cuda()
        d_out = torch.empty(len(g["sizes"]) * 120, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.map_to_curve_device(curve, d_u.data_ptr(), total, d_pts.data_ptr())
        torch.cuda.synchronize()
        groups[curve] = (g["sizes"], d_sc, d_pts, d_out)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def once():
        for curve, (sizes, d_sc, d_pts, d_out) in groups.items():
            ctx.msm_batch_device(curve, sizes, d_sc.data_ptr(), d_pts.data_ptr(), d_out.data_ptr(),
                                 hs.FMT_JACOBIAN51)
        stream.synchronize()

    for _ in range(2):
        once()
    t0 = time.perf_counter()
    for _ in range(reps):
        once()
    ms = (time.perf_counter() - t0) / max(1, reps) * 1e3
    print(json.dumps({"msms": int(len(bs["sizes"])), "points": int(sum(bs["sizes"])), "ms_per_batch": ms,
                      "launches": ctx.launches}))
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
