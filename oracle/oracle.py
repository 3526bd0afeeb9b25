"""ctypes binding of the C oracle (hs_oracle.c) -- TEST INFRASTRUCTURE ONLY.

The oracle is the checker for the GPU product: only the test suite, the smoke
check and the CPU-baseline leg of bench.py load it.  Formats (little endian):
scalars n*32 bytes, affine points n*64 bytes (x||y canonical, zeros =
identity), Jacobian points n*96 bytes (X||Y||Z), encoded points 32 bytes.
"""

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
HELIOS, SELENE = 0, 1
FIELD_P, FIELD_Q = 0, 1
CURVE_ID = {"helios": HELIOS, "selene": SELENE}

_lib = None


def build(force: bool = False) -> Path:
    """Compile hs_oracle.c into oracle/liboracle.so (gcc, no other deps)."""
    src = [HERE / "hs_oracle.c", HERE / "hs_field_impl.h", HERE / "hs_curve_impl.h", HERE / "hs_oracle.h"]
    if force or not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in src):
        subprocess.check_call(["make", "-C", str(HERE), "liboracle.so"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        c = ctypes
        u8p, sz = c.c_void_p, c.c_size_t
        sig = {
            "hso_msm": [c.c_int, u8p, u8p, u8p, sz, c.c_int],
            "hso_msm_affine_out": [c.c_int, u8p, u8p, u8p, u8p, sz, c.c_int],
            "hso_msm_jac": [c.c_int, u8p, u8p, u8p, sz, c.c_int],
            "hso_pippenger_w": [c.c_int, u8p, u8p, u8p, sz, c.c_int, c.c_int],
            "hso_msm_naive": [c.c_int, u8p, u8p, u8p, sz],
            "hso_msm_mt": [c.c_int, u8p, u8p, u8p, sz, c.c_int],
            "hso_msm_many": [c.c_int, u8p, u8p, u8p, u8p, sz, c.c_int],
            "hso_pedersen": [c.c_int, u8p, u8p, u8p, u8p, u8p, sz, c.c_int],
            "hso_map_to_curve": [c.c_int, u8p, u8p, sz],
            "hso_map_to_curve_mt": [c.c_int, u8p, u8p, sz, c.c_int],
            "hso_decompress": [c.c_int, u8p, u8p, sz],
            "hso_compress": [c.c_int, u8p, u8p, sz],
            "hso_compress_jac": [c.c_int, u8p, u8p, sz],
            "hso_batch_invert": [c.c_int, u8p, u8p, sz],
            "hso_batch_to_affine": [c.c_int, u8p, u8p, sz],
            "hso_scalar_mul": [c.c_int, u8p, u8p, u8p],
            "hso_point_add": [c.c_int, u8p, u8p, u8p],
            "hso_fe51_to_bytes": [c.c_int, u8p, u8p],
        }
        for name, args in sig.items():
            f = getattr(_lib, name)
            f.argtypes = args
            f.restype = c.c_int
    return _lib


def _buf(a) -> np.ndarray:
    arr = np.ascontiguousarray(np.frombuffer(bytes(a), dtype=np.uint8) if isinstance(a, (bytes, bytearray)) else a,
                               dtype=np.uint8)
    return arr


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _cid(curve) -> int:
    return CURVE_ID[curve] if isinstance(curve, str) else int(curve)


def msm(curve, scalars, points64, keep_carry=True) -> bytes:
    """Reference-restated MSM; keep_carry=False reproduces the reference exactly (w=8 defect)."""
    s, p = _buf(scalars), _buf(points64)
    n = s.size // 32
    assert p.size == 64 * n
    out = np.zeros(32, np.uint8)
    rc = lib().hso_msm(_cid(curve), _p(out), _p(s), _p(p), n, int(bool(keep_carry)))
    assert rc == 0
    return out.tobytes()


def msm_affine(curve, scalars, points64) -> tuple:
    s, p = _buf(scalars), _buf(points64)
    n = s.size // 32
    o32, o64 = np.zeros(32, np.uint8), np.zeros(64, np.uint8)
    assert lib().hso_msm_affine_out(_cid(curve), _p(o32), _p(o64), _p(s), _p(p), n, 1) == 0
    return o32.tobytes(), o64.tobytes()


def msm_jac(curve, scalars, jac96, keep_carry=True) -> bytes:
    s, p = _buf(scalars), _buf(jac96)
    n = s.size // 32
    assert p.size == 96 * n
    out = np.zeros(32, np.uint8)
    assert lib().hso_msm_jac(_cid(curve), _p(out), _p(s), _p(p), n, int(bool(keep_carry))) == 0
    return out.tobytes()


def pippenger_w(curve, scalars, points64, w, keep_carry=True) -> bytes:
    s, p = _buf(scalars), _buf(points64)
    out = np.zeros(32, np.uint8)
    assert lib().hso_pippenger_w(_cid(curve), _p(out), _p(s), _p(p), s.size // 32, w, int(bool(keep_carry))) == 0
    return out.tobytes()


def msm_naive(curve, scalars, points64) -> bytes:
    s, p = _buf(scalars), _buf(points64)
    out = np.zeros(32, np.uint8)
    assert lib().hso_msm_naive(_cid(curve), _p(out), _p(s), _p(p), s.size // 32) == 0
    return out.tobytes()


def msm_mt(curve, scalars, points64, nthreads) -> bytes:
    s, p = _buf(scalars), _buf(points64)
    out = np.zeros(32, np.uint8)
    assert lib().hso_msm_mt(_cid(curve), _p(out), _p(s), _p(p), s.size // 32, int(nthreads)) == 0
    return out.tobytes()


def msm_many(curve, scalars, points64, sizes, nthreads=None) -> list:
    """Independent exact-mode MSMs back to back (MSM i takes sizes[i] scalars and
    points after those of MSM i-1), on a pool of host threads; 32-byte results."""
    s, p = _buf(scalars), _buf(points64)
    sz = np.ascontiguousarray(np.asarray(sizes, dtype=np.uint64))
    assert s.size // 32 == int(sz.sum()) and p.size // 64 == int(sz.sum())
    out = np.zeros(32 * sz.size, np.uint8)
    rc = lib().hso_msm_many(_cid(curve), _p(out), _p(s), _p(p), _p(sz), sz.size,
                            int(nthreads or default_threads()))
    assert rc == 0
    return [out[32 * i:32 * (i + 1)].tobytes() for i in range(sz.size)]


def pedersen(curve, blinding, H64, values, gens64, keep_carry=True) -> bytes:
    b, h, v, g = _buf(blinding), _buf(H64), _buf(values), _buf(gens64)
    out = np.zeros(32, np.uint8)
    assert lib().hso_pedersen(_cid(curve), _p(out), _p(b), _p(h), _p(v), _p(g), v.size // 32,
                              int(bool(keep_carry))) == 0
    return out.tobytes()


def map_to_curve(curve, us) -> np.ndarray:
    u = _buf(us)
    n = u.size // 32
    out = np.zeros(64 * n, np.uint8)
    assert lib().hso_map_to_curve(_cid(curve), _p(out), _p(u), n) == 0
    return out


def map_to_curve_mt(curve, us, nthreads) -> np.ndarray:
    u = _buf(us)
    n = u.size // 32
    out = np.zeros(64 * n, np.uint8)
    assert lib().hso_map_to_curve_mt(_cid(curve), _p(out), _p(u), n, int(nthreads)) == 0
    return out


def decompress(curve, enc) -> tuple:
    e = _buf(enc)
    n = e.size // 32
    out = np.zeros(64 * n, np.uint8)
    bad = lib().hso_decompress(_cid(curve), _p(out), _p(e), n)
    return out, bad


def compress(curve, pts64) -> np.ndarray:
    p = _buf(pts64)
    n = p.size // 64
    out = np.zeros(32 * n, np.uint8)
    assert lib().hso_compress(_cid(curve), _p(out), _p(p), n) == 0
    return out


def compress_jac(curve, jac96) -> np.ndarray:
    p = _buf(jac96)
    n = p.size // 96
    out = np.zeros(32 * n, np.uint8)
    assert lib().hso_compress_jac(_cid(curve), _p(out), _p(p), n) == 0
    return out


def batch_invert(field, elems) -> np.ndarray:
    e = _buf(elems)
    out = np.zeros(e.size, np.uint8)
    assert lib().hso_batch_invert(int(field), _p(out), _p(e), e.size // 32) == 0
    return out


def batch_to_affine(curve, jac96) -> np.ndarray:
    j = _buf(jac96)
    n = j.size // 96
    out = np.zeros(64 * n, np.uint8)
    assert lib().hso_batch_to_affine(_cid(curve), _p(out), _p(j), n) == 0
    return out


def scalar_mul(curve, scalar, pt64) -> bytes:
    s, p = _buf(scalar), _buf(pt64)
    out = np.zeros(64, np.uint8)
    assert lib().hso_scalar_mul(_cid(curve), _p(out), _p(s), _p(p)) == 0
    return out.tobytes()


def point_add(curve, a64, b64) -> bytes:
    a, b = _buf(a64), _buf(b64)
    out = np.zeros(64, np.uint8)
    assert lib().hso_point_add(_cid(curve), _p(out), _p(a), _p(b)) == 0
    return out.tobytes()


def fe51_to_bytes(field, limbs) -> bytes:
    l = np.ascontiguousarray(np.asarray(limbs, dtype=np.uint64))
    out = np.zeros(32, np.uint8)
    assert lib().hso_fe51_to_bytes(int(field), _p(out), l.ctypes.data_as(ctypes.c_void_p)) == 0
    return out.tobytes()


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)
