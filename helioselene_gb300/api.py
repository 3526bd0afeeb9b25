"""Host API over the C ABI: a device context plus mirrors of the reference's
point API for this path (include/helioselene_point.h:113-174):

    HeliosPoint.multi_scalar_mul(scalars, points)       (api_point.cpp:98-116)
    HeliosPoint.pedersen_commit(r, H, values, gens)     (api_point.cpp:118-144)
    HeliosPoint.map_to_curve(u)                         (api_point.cpp:146-151)
    point.to_bytes()                                    (api_point.cpp:66-71)
    helios_batch_to_affine(points)                      (helios/include/helios_batch_affine.h:55)

and the Selene twins.  Points are held in the reference's own layout
(helios_jacobian: three radix-2^51 five-limb integers, 120 bytes).  Every
computation runs on the GPU through libhelioselene_gb300.so.
"""

from __future__ import annotations

import ctypes
import threading
from typing import Iterable, List, Sequence

import numpy as np

from . import _lib as L


def _u8(a) -> np.ndarray:
    if isinstance(a, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(a), dtype=np.uint8)
    arr = np.ascontiguousarray(a)
    if arr.dtype != np.uint8:
        arr = arr.view(np.uint8)
    return arr.reshape(-1)


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """One device, one CUDA stream, one grow-only workspace (hs_context)."""

    def __init__(self, device: int = 0):
        self._lib = L.load()
        h = ctypes.c_void_p()
        rc = self._lib.hs_context_create(ctypes.byref(h), int(device))
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_context_create: " + (self._lib.hs_last_error(None) or b"").decode())
        self._h = h
        self.device = device

    # -- lifetime --
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hs_context_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- plumbing --
    @property
    def handle(self):
        return self._h

    def _check(self, rc: int, what: str) -> None:
        if rc != L.HS_OK:
            msg = (self._lib.hs_last_error(self._h) or b"").decode()
            raise L.HsError(rc, f"{what}: {self._lib.hs_strerror(rc).decode()} {msg}")

    @property
    def launches(self) -> int:
        return int(self._lib.hs_context_launches(self._h))

    @property
    def stream(self) -> int:
        return int(self._lib.hs_context_stream(self._h) or 0)

    def set_window(self, curve: int, n_min: int, n_max: int, window: int, ba_rounds: int = -1) -> None:
        """window width (and optionally batch-affine rounds) for MSMs of n_min..n_max points; window 0 clears"""
        self._check(self._lib.hs_context_set_rule(self._h, curve, n_min, n_max, window, int(ba_rounds)),
                    "set_window")

    def set_graphs(self, on: bool) -> None:
        self._check(self._lib.hs_context_set_graphs(self._h, int(on)), "set_graphs")

    def set_priority(self, high: bool) -> None:
        """new context stream of the greatest (or default) priority; stream handle changes"""
        self._check(self._lib.hs_context_set_priority(self._h, int(bool(high))), "set_priority")

    def set_split(self, min_points: int) -> None:
        """single MSMs of >= min_points run as two window halves on two streams (0: off)"""
        self._check(self._lib.hs_context_set_split(self._h, int(min_points)), "set_split")

    def set_batch_affine(self, rounds: int, min_entries: int = 1 << 21, curve: int = None) -> None:
        """bucket accumulation by `rounds` rounds of batch-affine additions for plans of at
        least min_entries entries (0: XYZZ mixed additions throughout; -1: the library's
        defaults), for one curve or both"""
        for c in ((L.HELIOS, L.SELENE) if curve is None else (curve,)):
            self._check(self._lib.hs_context_set_batch_affine(self._h, c, int(rounds), int(min_entries)),
                        "set_batch_affine")

    def default_batch_affine(self) -> None:
        """the library's default accumulation forms: one batch-affine round on Helios and two
        on Selene, except fixed-base commitments and single MSMs from host buffers, which
        take none on Helios and one on Selene"""
        self.set_batch_affine(-1)

    # -- instrumentation --
    def profile(self, on: bool = True) -> None:
        self._check(self._lib.hs_profile_enable(self._h, int(on)), "hs_profile_enable")

    def profile_read(self, reset: bool = True) -> dict:
        ms, launches, entries = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._lib.hs_profile_read(self._h, ctypes.byref(ms), ctypes.byref(launches),
                                              ctypes.byref(entries), int(reset)), "hs_profile_read")
        return {"accumulate_ms": ms.value, "accumulate_launches": launches.value, "entries": entries.value}

    def measure_imad_peak(self) -> float:
        v = ctypes.c_double()
        self._check(self._lib.hs_measure_imad_peak(self._h, ctypes.byref(v)), "hs_measure_imad_peak")
        return v.value

    def measure_imad_rates(self) -> dict:
        """the probes behind measure_imad_peak, instructions per second over the device"""
        r = (ctypes.c_double * 4)()
        self._check(self._lib.hs_measure_imad_rates(self._h, r), "hs_measure_imad_rates")
        return {"mad_lo_hi": r[0], "mad_wide": r[1], "mad_lo": r[2], "mad_hi": r[3]}

    def field_op(self, field: int, op: int, a, b=None) -> np.ndarray:
        """Element-wise device field arithmetic (0 mul, 1 sqr, 2 add, 3 sub, 4 canon, 5 inv, 6 neg;
        the window combination's lane-sliced form: 7 mul, 8 (a - b)(a + b), 9 a^(2^32), 10 round trip)."""
        x = _u8(a)
        y = _u8(b) if b is not None else x
        n = x.size // 32
        out = np.zeros(32 * n, np.uint8)
        self._check(self._lib.hs_field_op(self._h, field, op, _ptr(x), _ptr(y), n, _ptr(out)), "hs_field_op")
        return out

    # -- MSM --
    def msm(self, curve: int, scalars, points, point_fmt: int = L.FMT_AFFINE,
            out_fmt: int = L.FMT_COMPRESSED) -> bytes:
        s, p = _u8(scalars), _u8(points)
        n = s.size // 32
        if s.size != 32 * n or p.size != L.FMT_BYTES[point_fmt] * n:
            raise ValueError("scalars / points sizes do not match")
        out = np.zeros(L.FMT_BYTES[out_fmt], np.uint8)
        self._check(self._lib.hs_msm(self._h, curve, _ptr(s), _ptr(p), point_fmt, n, _ptr(out), out_fmt), "hs_msm")
        return out.tobytes()

    def msm_device(self, curve: int, d_scalars: int, d_points: int, n: int, d_out: int,
                   out_fmt: int = L.FMT_JACOBIAN51) -> None:
        self._check(self._lib.hs_msm_device(self._h, curve, ctypes.c_void_p(d_scalars), ctypes.c_void_p(d_points),
                                            n, ctypes.c_void_p(d_out), out_fmt), "hs_msm_device")

    def pedersen(self, curve: int, blinding, H, values, generators, point_fmt: int = L.FMT_AFFINE,
                 out_fmt: int = L.FMT_COMPRESSED) -> bytes:
        b, h, v, g = _u8(blinding), _u8(H), _u8(values), _u8(generators)
        n = v.size // 32
        out = np.zeros(L.FMT_BYTES[out_fmt], np.uint8)
        self._check(self._lib.hs_pedersen(self._h, curve, _ptr(b), _ptr(h), _ptr(v), _ptr(g), point_fmt, n,
                                          _ptr(out), out_fmt), "hs_pedersen")
        return out.tobytes()

    def msm_batch(self, items: Sequence[tuple], point_fmt: int = L.FMT_AFFINE,
                  out_fmt: int = L.FMT_COMPRESSED) -> List[bytes]:
        """items: (curve, scalars, points) triples; returns one output per MSM."""
        keep, descs = [], (L.hs_msm_desc * max(1, len(items)))()
        outs = []
        for i, (curve, sc, pts) in enumerate(items):
            s, p = _u8(sc), _u8(pts)
            o = np.zeros(L.FMT_BYTES[out_fmt], np.uint8)
            keep += [s, p]
            outs.append(o)
            descs[i].curve, descs[i].n = curve, s.size // 32
            descs[i].scalars, descs[i].points, descs[i].out = s.ctypes.data, p.ctypes.data, o.ctypes.data
        self._check(self._lib.hs_msm_batch(self._h, descs, len(items), point_fmt, out_fmt), "hs_msm_batch")
        return [o.tobytes() for o in outs]

    def msm_batch_device(self, curve: int, sizes: Sequence[int], d_scalars: int, d_points: int, d_out: int,
                         out_fmt: int = L.FMT_JACOBIAN51) -> None:
        """Batched MSMs on one curve over concatenated device arrays (hs_msm_batch_device)."""
        sz = np.ascontiguousarray(np.asarray(sizes, dtype=np.uint64))
        self._check(self._lib.hs_msm_batch_device(self._h, curve, sz.ctypes.data_as(ctypes.c_void_p), len(sizes),
                                                  ctypes.c_void_p(d_scalars), ctypes.c_void_p(d_points),
                                                  ctypes.c_void_p(d_out), out_fmt), "hs_msm_batch_device")

    # -- conversions --
    def batch_to_affine(self, curve: int, jac51, out_fmt: int = L.FMT_AFFINE) -> np.ndarray:
        j = _u8(jac51)
        n = j.size // 120
        out = np.zeros(n * L.FMT_BYTES[out_fmt], np.uint8)
        self._check(self._lib.hs_batch_to_affine(self._h, curve, _ptr(j), n, _ptr(out), out_fmt),
                    "hs_batch_to_affine")
        return out

    def compress(self, curve: int, points, in_fmt: int) -> np.ndarray:
        p = _u8(points)
        n = p.size // L.FMT_BYTES[in_fmt]
        out = np.zeros(32 * n, np.uint8)
        self._check(self._lib.hs_compress(self._h, curve, _ptr(p), in_fmt, n, _ptr(out)), "hs_compress")
        return out

    def scalar_mul(self, curve: int, scalars, points, point_fmt: int = L.FMT_AFFINE,
                   out_fmt: int = L.FMT_COMPRESSED) -> np.ndarray:
        """out[i] = scalars[i] * points[i], variable time (hs_scalar_mul); n records of out_fmt"""
        s, p = _u8(scalars), _u8(points)
        n = s.size // 32
        out = np.zeros(n * L.FMT_BYTES[out_fmt], np.uint8)
        self._check(self._lib.hs_scalar_mul(self._h, curve, _ptr(s), _ptr(p), point_fmt, n, _ptr(out), out_fmt),
                    "hs_scalar_mul")
        return out

    def scalar_mul_device(self, curve: int, d_scalars: int, d_points: int, n: int, d_out: int,
                          out_fmt: int = L.FMT_JACOBIAN51) -> None:
        self._check(self._lib.hs_scalar_mul_device(self._h, curve, ctypes.c_void_p(d_scalars),
                                                   ctypes.c_void_p(d_points), n, ctypes.c_void_p(d_out), out_fmt),
                    "hs_scalar_mul_device")

    def decompress(self, curve: int, encodings, out_fmt: int = L.FMT_AFFINE, check: bool = True):
        """32-byte encodings -> points in out_fmt and a validity mask (hs_decompress).
        With check=False invalid encodings come back as the identity instead of raising."""
        e = _u8(encodings)
        n = e.size // 32
        out = np.zeros(n * L.FMT_BYTES[out_fmt], np.uint8)
        valid = np.zeros(n, np.uint8)
        rc = self._lib.hs_decompress(self._h, curve, _ptr(e), n, _ptr(out), out_fmt, _ptr(valid))
        if rc != L.HS_EINVAL or check:
            self._check(rc, "hs_decompress")
        return out, valid.astype(bool)

    def decompress_device(self, curve: int, d_in: int, n: int, d_out: int, d_valid: int) -> None:
        self._check(self._lib.hs_decompress_device(self._h, curve, ctypes.c_void_p(d_in), n, ctypes.c_void_p(d_out),
                                                   ctypes.c_void_p(d_valid)), "hs_decompress_device")

    def map_to_curve(self, curve: int, u, out_fmt: int = L.FMT_AFFINE) -> np.ndarray:
        uu = _u8(u)
        n = uu.size // 32
        out = np.zeros(n * L.FMT_BYTES[out_fmt], np.uint8)
        self._check(self._lib.hs_map_to_curve(self._h, curve, _ptr(uu), n, _ptr(out), out_fmt), "hs_map_to_curve")
        return out

    def map_to_curve_device(self, curve: int, d_u: int, n: int, d_out: int) -> None:
        self._check(self._lib.hs_map_to_curve_device(self._h, curve, ctypes.c_void_p(d_u), n,
                                                     ctypes.c_void_p(d_out)), "hs_map_to_curve_device")


class FixedBase:
    """Resident generator set with device window tables (hs_fixed_base_*):
    commitments r*H + sum v_i G_i over the same generators."""

    def __init__(self, ctx: Context, curve: int, generators, H=None, point_fmt: int = L.FMT_AFFINE, window: int = 0):
        self.ctx, self.curve = ctx, curve
        g = _u8(generators)
        self.n = g.size // L.FMT_BYTES[point_fmt]
        h = _u8(H) if H is not None else None
        fb = ctypes.c_void_p()
        ctx._check(ctx._lib.hs_fixed_base_create(ctx.handle, curve, _ptr(g), point_fmt, self.n,
                                                 None if h is None else _ptr(h), window, ctypes.byref(fb)),
                   "hs_fixed_base_create")
        self._fb = fb
        self.has_H = H is not None
        w, tb = ctypes.c_int(), ctypes.c_size_t()
        ctx._lib.hs_fixed_base_info(fb, ctypes.byref(w), ctypes.byref(tb))
        self.window, self.table_bytes = w.value, tb.value

    def commit(self, values, blindings=None, out_fmt: int = L.FMT_COMPRESSED) -> List[bytes]:
        v = _u8(values)
        count = v.size // (32 * self.n) if self.n else (len(blindings) // 32 if blindings is not None else 0)
        b = _u8(blindings) if blindings is not None else None
        out = np.zeros(count * L.FMT_BYTES[out_fmt], np.uint8)
        self.ctx._check(self.ctx._lib.hs_fixed_base_commit(self.ctx.handle, self._fb, _ptr(v),
                                                           None if b is None else _ptr(b), count, _ptr(out),
                                                           out_fmt), "hs_fixed_base_commit")
        ob = L.FMT_BYTES[out_fmt]
        return [out[ob * i:ob * (i + 1)].tobytes() for i in range(count)]

    def commit_device(self, d_scalars: int, count: int, d_out: int, out_fmt: int = L.FMT_JACOBIAN51) -> None:
        self.ctx._check(self.ctx._lib.hs_fixed_base_commit_device(self.ctx.handle, self._fb,
                                                                  ctypes.c_void_p(d_scalars), count,
                                                                  ctypes.c_void_p(d_out), out_fmt),
                        "hs_fixed_base_commit_device")

    def close(self) -> None:
        if getattr(self, "_fb", None):
            self.ctx._lib.hs_fixed_base_destroy(self._fb)
            self._fb = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching MSM server (hs_server_*): submit requests as they
    arrive, wait for each; the native scheduler batches whatever is queued onto
    free slots within the HBM budget."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int = 0, max_batch_points: int = 0,
                 max_batch_msms: int = 0, out_fmt: int = L.FMT_COMPRESSED):
        self._lib = L.load()
        cfg = L.hs_server_config(device, slots, hbm_budget, max_batch_points, max_batch_msms, out_fmt)
        h = ctypes.c_void_p()
        rc = self._lib.hs_server_create(ctypes.byref(h), ctypes.byref(cfg))
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_server_create")
        self._h = h
        self.out_bytes = L.FMT_BYTES[out_fmt]
        self._live = {}

    def set_pool(self, curve: int, affine_points) -> None:
        """resident base pool of one curve (and, unless its pool window is 0,
        the table of window multiples that requests with pooled bases only are
        computed from)"""
        p = _u8(affine_points)
        rc = self._lib.hs_server_set_pool(self._h, curve, _ptr(p), p.size // 64)
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_server_set_pool")

    def set_pool_window(self, curve: int, window: int) -> None:
        """window width of the curve's pool table from the next set_pool (4..16;
        0: no table, pooled bases gathered as variable bases)"""
        rc = self._lib.hs_server_set_pool_window(self._h, curve, int(window))
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_server_set_pool_window")

    def set_window(self, curve: int, n_min: int, n_max: int, window: int) -> None:
        """window rule for every slot's batches (hs_server_set_window; window 0 clears)"""
        rc = self._lib.hs_server_set_window(self._h, curve, int(n_min), int(n_max), int(window))
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_server_set_window")

    def submit(self, curve: int, scalars, pool_idx=None, fresh_points=None) -> int:
        s = _u8(scalars)
        idx = np.ascontiguousarray(pool_idx, dtype=np.uint32) if pool_idx is not None else None
        fr = _u8(fresh_points) if fresh_points is not None else None
        out = np.zeros(self.out_bytes, np.uint8)
        req = L.hs_request(curve, 0 if idx is None else idx.size, None if idx is None else idx.ctypes.data,
                           0 if fr is None else fr.size // 64, None if fr is None else fr.ctypes.data,
                           s.ctypes.data, out.ctypes.data)
        t = ctypes.c_uint64()
        rc = self._lib.hs_server_submit(self._h, ctypes.byref(req), ctypes.byref(t))
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_server_submit")
        self._live[t.value] = (s, idx, fr, out)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000):
        """-> (result bytes, latency_ms from submit to completion)"""
        lat = ctypes.c_double()
        rc = self._lib.hs_server_wait(self._h, ticket, timeout_ms, ctypes.byref(lat))
        if rc == L.HS_ETIMEDOUT:
            raise TimeoutError(f"request {ticket} not done after {timeout_ms} ms")
        bufs = self._live.pop(ticket)
        if rc != L.HS_OK:
            raise L.HsError(rc, "hs_server_wait")
        return bufs[3].tobytes(), lat.value

    def stats(self) -> dict:
        st = L.hs_server_stats()
        self._lib.hs_server_get_stats(self._h, ctypes.byref(st))
        return {f: int(getattr(st, f)) for f, _ in L.hs_server_stats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hs_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None
_default_lock = threading.Lock()


def default_context() -> Context:
    global _default
    with _default_lock:
        if _default is None:
            _default = Context(0)
        return _default


# ---------------------------------------------------------------------------
# radix-2^51 packing (pure integer repacking, the reference's fp_fe layout)
# ---------------------------------------------------------------------------
M51 = (1 << 51) - 1


def int_to_fe51(v: int) -> List[int]:
    return [(v >> (51 * i)) & M51 for i in range(5)]


def fe51_to_int(limbs: Iterable[int]) -> int:
    return sum(int(l) << (51 * i) for i, l in enumerate(limbs))


def jac51_from_ints(X: int, Y: int, Z: int) -> bytes:
    return np.array(int_to_fe51(X) + int_to_fe51(Y) + int_to_fe51(Z), dtype=np.uint64).tobytes()


def affine64_to_jac51(aff: np.ndarray) -> np.ndarray:
    """Canonical affine x||y (64 bytes each, zeros = identity) -> helios_jacobian records (Z = 1)."""
    a = _u8(aff).reshape(-1, 64)
    out = np.zeros((a.shape[0], 15), np.uint64)
    for i in range(a.shape[0]):
        x = int.from_bytes(a[i, :32].tobytes(), "little")
        y = int.from_bytes(a[i, 32:].tobytes(), "little")
        if x == 0 and y == 0:
            out[i] = int_to_fe51(1) + int_to_fe51(1) + int_to_fe51(0)
        else:
            out[i] = int_to_fe51(x) + int_to_fe51(y) + int_to_fe51(1)
    return out.reshape(-1).view(np.uint8)


# ---------------------------------------------------------------------------
# mirrors of HeliosPoint / SelenePoint for the MSM path
# ---------------------------------------------------------------------------
class _PointBase:
    CURVE = L.HELIOS

    def __init__(self, jac51: bytes):
        if len(jac51) != 120:
            raise ValueError("a point is one 120-byte helios_jacobian / selene_jacobian record")
        self.jac51 = bytes(jac51)

    @classmethod
    def identity(cls):
        return cls(jac51_from_ints(1, 1, 0))

    @classmethod
    def from_bytes(cls, data: bytes, ctx: Context = None):
        """Decode a 32-byte encoding on the device; None when the reference rejects
        it (HeliosPoint::from_bytes, src/api_point.cpp:58-64)."""
        ctx = ctx or default_context()
        out, valid = ctx.decompress(cls.CURVE, bytes(data), L.FMT_JACOBIAN51, check=False)
        return cls(out.tobytes()) if valid[0] else None

    @classmethod
    def from_affine_bytes(cls, aff64) -> "_PointBase":
        return cls(affine64_to_jac51(np.asarray(_u8(aff64))).tobytes())

    def is_identity(self) -> bool:
        z = np.frombuffer(self.jac51, dtype=np.uint64)[10:15]
        return self.to_bytes() == bytes(32) if z.any() else True

    def to_bytes(self, ctx: Context = None) -> bytes:
        ctx = ctx or default_context()
        return ctx.compress(self.CURVE, self.jac51, L.FMT_JACOBIAN51).tobytes()

    def __eq__(self, other) -> bool:
        return type(self) is type(other) and self.to_bytes() == other.to_bytes()

    def __hash__(self):
        return hash(self.to_bytes())

    @classmethod
    def multi_scalar_mul(cls, scalars: Sequence[bytes], points: Sequence["_PointBase"], ctx: Context = None):
        """Sum scalars[i] * points[i]; n == 0 gives the identity (api_point.cpp:100-101)."""
        ctx = ctx or default_context()
        if len(scalars) == 0 or len(points) == 0:
            return cls.identity()
        s = b"".join(bytes(x) for x in scalars)
        p = b"".join(pt.jac51 for pt in points)
        return cls(ctx.msm(cls.CURVE, s, p, L.FMT_JACOBIAN51, L.FMT_JACOBIAN51))

    @classmethod
    def pedersen_commit(cls, blinding: bytes, H: "_PointBase", values: Sequence[bytes],
                        generators: Sequence["_PointBase"], ctx: Context = None):
        """blinding*H + sum values[i]*generators[i] (api_point.cpp:118-144; n == 0 -> identity)."""
        ctx = ctx or default_context()
        if len(values) == 0 or len(generators) == 0:
            return cls.identity()
        v = b"".join(bytes(x) for x in values)
        g = b"".join(pt.jac51 for pt in generators)
        return cls(ctx.pedersen(cls.CURVE, bytes(blinding), H.jac51, v, g, L.FMT_JACOBIAN51, L.FMT_JACOBIAN51))

    def scalar_mul_vartime(self, scalar: bytes, ctx: Context = None):
        """scalar * self, variable time, for public scalars (helios_scalarmult_vartime,
        helios/include/helios_scalarmult_vartime.h:39-57)"""
        ctx = ctx or default_context()
        return type(self)(ctx.scalar_mul(self.CURVE, bytes(scalar), self.jac51, L.FMT_JACOBIAN51,
                                         L.FMT_JACOBIAN51).tobytes())

    @classmethod
    def map_to_curve(cls, u: bytes, ctx: Context = None):
        ctx = ctx or default_context()
        return cls(ctx.map_to_curve(cls.CURVE, bytes(u), L.FMT_JACOBIAN51).tobytes())


class HeliosPoint(_PointBase):
    CURVE = L.HELIOS


class SelenePoint(_PointBase):
    CURVE = L.SELENE


def _batch_to_affine(curve: int, points: Sequence[_PointBase], ctx: Context = None) -> List[bytes]:
    ctx = ctx or default_context()
    if not points:
        return []
    out = ctx.batch_to_affine(curve, b"".join(p.jac51 for p in points), L.FMT_AFFINE)
    return [out[64 * i:64 * i + 64].tobytes() for i in range(len(points))]


def helios_batch_to_affine(points: Sequence[HeliosPoint], ctx: Context = None) -> List[bytes]:
    """Affine (x||y canonical bytes) of each point, identity -> zeros (helios_batch_affine.h:55-98)."""
    return _batch_to_affine(L.HELIOS, points, ctx)


def selene_batch_to_affine(points: Sequence[SelenePoint], ctx: Context = None) -> List[bytes]:
    return _batch_to_affine(L.SELENE, points, ctx)
