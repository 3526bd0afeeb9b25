"""The reference's MSM and Pedersen golden-vector checks (src/tests.cpp:6036-6142)
through the C++ point API of include/helioselene_gb300.hpp, in a program built
with g++ and linked against the library: decode with from_bytes, run
multi_scalar_mul / pedersen_commit on the GPU, compare to_bytes."""

import subprocess

import pytest

import _cpp

pytestmark = pytest.mark.gpu


def test_golden_vectors_through_the_cpp_point_api(tmp_path, golden):
    exe = _cpp.build_golden_program(tmp_path)
    n = _cpp.write_cases(golden, tmp_path / "cases.txt")
    r = subprocess.run([str(exe), str(tmp_path / "cases.txt")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ok = [ln for ln in r.stdout.splitlines() if ln.startswith("ok ")]
    assert len(ok) == n, r.stdout
