"""ctypes binding of libhelioselene_gb300.so (the C ABI in include/helioselene_gb300.h).

The shared library is the product; this module only loads it and declares the
signatures.  There is no fallback: if the library is missing the import of
any compute entry point raises.
"""

import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libhelioselene_gb300.so"

HS_OK, HS_EINVAL, HS_ENOMEM, HS_ECUDA, HS_ETIMEDOUT, HS_EBUSY, HS_ERANGE = 0, -1, -2, -3, -4, -5, -6
HELIOS, SELENE = 0, 1
FMT_JACOBIAN51, FMT_AFFINE51, FMT_AFFINE, FMT_COMPRESSED = 0, 1, 2, 3
FMT_BYTES = {FMT_JACOBIAN51: 120, FMT_AFFINE51: 80, FMT_AFFINE: 64, FMT_COMPRESSED: 32}


class HsError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what} (status {status})")
        self.status = status


class hs_msm_desc(ctypes.Structure):
    _fields_ = [("curve", ctypes.c_int), ("n", ctypes.c_size_t), ("scalars", ctypes.c_void_p),
                ("points", ctypes.c_void_p), ("out", ctypes.c_void_p)]


class hs_server_config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("slots", ctypes.c_int), ("hbm_budget", ctypes.c_size_t),
                ("max_batch_points", ctypes.c_size_t), ("max_batch_msms", ctypes.c_size_t), ("out_fmt", ctypes.c_int)]


class hs_request(ctypes.Structure):
    _fields_ = [("curve", ctypes.c_int), ("n_pool", ctypes.c_size_t), ("pool_idx", ctypes.c_void_p),
                ("n_fresh", ctypes.c_size_t), ("fresh_points", ctypes.c_void_p), ("scalars", ctypes.c_void_p),
                ("out", ctypes.c_void_p)]


class hs_server_stats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("max_batch_msms", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64),
                ("deferred", ctypes.c_uint64)]


# name -> (restype, argtypes); mirrors include/helioselene_gb300.h
_c = ctypes
_vp, _sz, _int = _c.c_void_p, _c.c_size_t, _c.c_int
SIGNATURES = {
    "hs_abi_version": (_int, []),
    "hs_strerror": (_c.c_char_p, [_int]),
    "hs_context_create": (_int, [_c.POINTER(_vp), _int]),
    "hs_context_destroy": (None, [_vp]),
    "hs_last_error": (_c.c_char_p, [_vp]),
    "hs_context_launches": (_c.c_uint64, [_vp]),
    "hs_context_stream": (_vp, [_vp]),
    "hs_context_set_window": (_int, [_vp, _int, _sz, _sz, _int]),
    "hs_context_set_graphs": (_int, [_vp, _int]),
    "hs_context_set_split": (_int, [_vp, _sz]),
    "hs_context_set_batch_affine": (_int, [_vp, _int, _int, _sz]),
    "hs_context_set_rule": (_int, [_vp, _int, _sz, _sz, _int, _int]),
    "hs_context_set_priority": (_int, [_vp, _int]),
    "hs_msm": (_int, [_vp, _int, _vp, _vp, _int, _sz, _vp, _int]),
    "hs_msm_device": (_int, [_vp, _int, _vp, _vp, _sz, _vp, _int]),
    "hs_pedersen": (_int, [_vp, _int, _vp, _vp, _vp, _vp, _int, _sz, _vp, _int]),
    "hs_batch_to_affine": (_int, [_vp, _int, _vp, _sz, _vp, _int]),
    "hs_compress": (_int, [_vp, _int, _vp, _int, _sz, _vp]),
    "hs_decompress": (_int, [_vp, _int, _vp, _sz, _vp, _int, _vp]),
    "hs_scalar_mul": (_int, [_vp, _int, _vp, _vp, _int, _sz, _vp, _int]),
    "hs_scalar_mul_device": (_int, [_vp, _int, _vp, _vp, _sz, _vp, _int]),
    "hs_decompress_device": (_int, [_vp, _int, _vp, _sz, _vp, _vp]),
    "hs_map_to_curve": (_int, [_vp, _int, _vp, _sz, _vp, _int]),
    "hs_map_to_curve_device": (_int, [_vp, _int, _vp, _sz, _vp]),
    "hs_msm_batch": (_int, [_vp, _c.POINTER(hs_msm_desc), _sz, _int, _int]),
    "hs_msm_batch_device": (_int, [_vp, _int, _vp, _sz, _vp, _vp, _vp, _int]),
    "hs_profile_enable": (_int, [_vp, _int]),
    "hs_profile_read": (_int, [_vp, _c.POINTER(_c.c_double), _c.POINTER(_c.c_uint64), _c.POINTER(_c.c_uint64),
                               _int]),
    "hs_measure_imad_peak": (_int, [_vp, _c.POINTER(_c.c_double)]),
    "hs_measure_imad_rates": (_int, [_vp, _c.POINTER(_c.c_double)]),
    "hs_field_op": (_int, [_vp, _int, _int, _vp, _vp, _sz, _vp]),
    "hs_fixed_base_create": (_int, [_vp, _int, _vp, _int, _sz, _vp, _int, _c.POINTER(_vp)]),
    "hs_fixed_base_commit": (_int, [_vp, _vp, _vp, _vp, _sz, _vp, _int]),
    "hs_fixed_base_commit_device": (_int, [_vp, _vp, _vp, _sz, _vp, _int]),
    "hs_fixed_base_info": (_int, [_vp, _c.POINTER(_int), _c.POINTER(_sz)]),
    "hs_fixed_base_destroy": (None, [_vp]),
    "hs_server_create": (_int, [_c.POINTER(_vp), _c.POINTER(hs_server_config)]),
    "hs_server_set_pool": (_int, [_vp, _int, _vp, _sz]),
    "hs_server_set_pool_window": (_int, [_vp, _int, _int]),
    "hs_server_set_window": (_int, [_vp, _int, _sz, _sz, _int]),
    "hs_server_submit": (_int, [_vp, _c.POINTER(hs_request), _c.POINTER(_c.c_uint64)]),
    "hs_server_wait": (_int, [_vp, _c.c_uint64, _int, _c.POINTER(_c.c_double)]),
    "hs_server_get_stats": (_int, [_vp, _c.POINTER(hs_server_stats)]),
    "hs_server_destroy": (None, [_vp]),
    "hs_msm_device_noalloc": (_int, [_int, _vp, _vp, _sz, _vp, _int, _vp]),
    "hs_msm_noalloc_scratch_bytes": (_sz, []),
    "hs_helios_msm_vartime": (None, [_vp, _vp, _vp, _sz]),
    "hs_selene_msm_vartime": (None, [_vp, _vp, _vp, _sz]),
    "hs_helios_scalarmult_vartime": (None, [_vp, _vp, _vp]),
    "hs_selene_scalarmult_vartime": (None, [_vp, _vp, _vp]),
    "hs_helios_pedersen_commit": (None, [_vp, _vp, _vp, _vp, _vp, _sz]),
    "hs_selene_pedersen_commit": (None, [_vp, _vp, _vp, _vp, _vp, _sz]),
    "hs_helios_batch_to_affine": (None, [_vp, _vp, _sz]),
    "hs_selene_batch_to_affine": (None, [_vp, _vp, _sz]),
}

_lib = None


def load(path: Path = LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not Path(path).exists():
            raise ImportError(f"{path} is missing: run helioselene_gb300.build.build() first "
                              "(there is no CPU implementation)")
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib
