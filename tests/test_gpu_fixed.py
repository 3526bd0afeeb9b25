"""Fixed-base commitments over resident window tables against the oracle's
Pedersen (helios/include/helios_pedersen.h:55-86 restated)."""

import numpy as np
import pytest

import oracle
from conftest import oracle_inputs

pytestmark = pytest.mark.gpu


def sparse_scalars(rng, count, n, bits=16):
    out = np.zeros((count, n, 32), np.uint8)
    for j in range(count):
        for i in range(n):
            v = 0
            for b in rng.choice(252, size=int(rng.integers(1, bits + 1)), replace=False):
                v |= 1 << int(b)
            out[j, i] = np.frombuffer(v.to_bytes(32, "little"), np.uint8)
    return out


@pytest.mark.parametrize("curve", [0, 1])
@pytest.mark.parametrize("window", [0, 8, 13, 20])
def test_fixed_base_pedersen(ctx, curve, window):
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import ORDER, random_scalars
    n, count = 300, 6
    _, gens, _ = oracle_inputs(curve, n + 1, seed=31 + curve)
    H, G = gens[n], gens[:n]
    rng = np.random.default_rng(window + 5)
    vals = random_scalars(rng, count * n, ORDER[curve]).reshape(count, n, 32)
    vals[1] = sparse_scalars(rng, 1, n)[0]          # sparse commitment (<= 16 set bits per scalar)
    vals[2, :50] = 0
    blinds = random_scalars(rng, count, ORDER[curve])
    blinds[3] = 0
    fb = hs.FixedBase(ctx, curve, G, H=H, window=window)
    try:
        got = fb.commit(vals, blinds)
        want = [oracle.pedersen(curve, blinds[j], H, vals[j], G) for j in range(count)]
        assert got == want
        # affine outputs (shared-inversion normalisation) encode to the same points
        aff = fb.commit(vals, blinds, out_fmt=hs.FMT_AFFINE)
        assert [oracle.compress(curve, a).tobytes() for a in aff] == want
    finally:
        fb.close()


@pytest.mark.parametrize("curve", [0, 1])
def test_fixed_base_without_H_and_device_api(ctx, curve):
    torch = pytest.importorskip("torch")
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import ORDER, random_scalars
    n, count = 2000, 5
    _, G, _ = oracle_inputs(curve, n, seed=77 + curve)
    G[10] = 0  # an identity generator in the set
    rng = np.random.default_rng(9)
    vals = random_scalars(rng, count * n, ORDER[curve]).reshape(count, n, 32)
    fb = hs.FixedBase(ctx, curve, G)
    try:
        want = [oracle.msm(curve, vals[j], G) for j in range(count)]
        assert fb.commit(vals) == want
        d_sc = torch.from_numpy(vals.reshape(-1).copy()).cuda()
        d_out = torch.zeros(count * 32, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        fb.commit_device(d_sc.data_ptr(), count, d_out.data_ptr(), hs.FMT_COMPRESSED)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        out = d_out.cpu().numpy().reshape(count, 32)
        assert [out[j].tobytes() for j in range(count)] == want
    finally:
        fb.close()


def test_fixed_base_refuses_blinding_without_H(ctx):
    import helioselene_gb300 as hs
    _, G, _ = oracle_inputs(0, 10, seed=1)
    fb = hs.FixedBase(ctx, 0, G)
    try:
        with pytest.raises(hs.HsError):
            fb.commit(np.zeros((1, 10, 32), np.uint8), np.zeros((1, 32), np.uint8))
    finally:
        fb.close()


@pytest.mark.parametrize("curve,n", [(1, 228), (1, 38), (0, 18)])
def test_tree_hash_layer_shapes(ctx, curve, n):
    """the FCMP++ tree-hash node shapes (src/benchmark_fcmpp.cpp:137-198): one
    layer = many MSMs over the same generators, each output taken to affine"""
    import helioselene_gb300 as hs
    from helioselene_gb300.workload import ORDER, random_scalars
    count = 40
    _, G, _ = oracle_inputs(curve, n, seed=300 + n)
    rng = np.random.default_rng(n)
    vals = random_scalars(rng, count * n, ORDER[curve]).reshape(count, n, 32)
    fb = hs.FixedBase(ctx, curve, G)
    try:
        aff = fb.commit(vals, out_fmt=hs.FMT_AFFINE)
        want = [oracle.msm(curve, vals[j], G) for j in range(count)]
        assert [oracle.compress(curve, a).tobytes() for a in aff] == want
        assert fb.commit(vals) == want
    finally:
        fb.close()
