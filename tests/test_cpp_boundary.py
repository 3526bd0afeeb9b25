"""The C++17 host layer (include/helioselene_gb300.hpp) compiles: against the
reference's own headers, where its point records must have the layout of the
C ABI's (static assertions) and every binding with the reference's signatures
and the adapters over helioselene::HeliosPoint / SelenePoint must build; and
standalone, as the golden-vector program the GPU test runs, linked against the
library.  CPU only: nothing runs on a device."""

import subprocess

import pytest

import _cpp


def test_header_compiles_against_the_reference_headers(tmp_path):
    ref = _cpp.reference_root()
    if ref is None:
        pytest.skip("the helioselene checkout is not present (HELIOSELENE_REF)")
    r = subprocess.run([_cpp.gxx(), "-std=c++17", "-Wall", "-Wextra", "-Werror", "-c", f"-I{_cpp.INCLUDE}",
                        *_cpp.reference_includes(ref), str(_cpp.CPP / "reference_types.cpp"),
                        "-o", str(tmp_path / "reference_types.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_layout_mismatch_is_rejected(tmp_path):
    """the layout check fires on a record of another layout (planted here, in a test TU)"""
    src = tmp_path / "bad.cpp"
    src.write_text('#include "helioselene_gb300.hpp"\n'
                   "struct other { unsigned long long X[4], Y[5], Z[5]; };\n"
                   "static_assert(helioselene_gb300::jacobian_layout_matches<other>(), \"layout\");\n")
    r = subprocess.run([_cpp.gxx(), "-std=c++17", "-c", f"-I{_cpp.INCLUDE}", str(src), "-o", str(tmp_path / "b.o")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "layout" in r.stderr


def test_golden_program_builds(tmp_path, golden):
    from helioselene_gb300 import build
    build.build()
    exe = _cpp.build_golden_program(tmp_path)
    assert exe.exists()
    assert _cpp.write_cases(golden, tmp_path / "cases.txt") >= 14
