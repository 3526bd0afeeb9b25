"""The C ABI library loads and exports every entry point include/*.h declares.
CPU only: nothing here launches device work."""

import ctypes
import re

import pytest

from conftest import ROOT

HEADER_DIR = ROOT / "include"


def declared_functions():
    names = set()
    for h in HEADER_DIR.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(hs_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from helioselene_gb300 import build
    path = build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("hs_msm", "hs_msm_device", "hs_pedersen", "hs_batch_to_affine", "hs_compress",
                     "hs_map_to_curve", "hs_msm_batch", "hs_helios_msm_vartime", "hs_selene_msm_vartime"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_the_header():
    from helioselene_gb300 import _lib
    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"


def test_host_only_calls(lib):
    lib.hs_abi_version.restype = ctypes.c_int
    assert lib.hs_abi_version() == 1
    lib.hs_strerror.restype = ctypes.c_char_p
    assert lib.hs_strerror(-1) == b"invalid argument"
    # argument validation happens before any device call
    lib.hs_msm.restype = ctypes.c_int
    assert lib.hs_msm(None, 0, None, None, 0, 0, None, 0) == -1
    lib.hs_context_create.restype = ctypes.c_int
    assert lib.hs_context_create(None, 0) == -1
