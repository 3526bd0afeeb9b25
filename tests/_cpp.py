"""Build helpers for the C++ boundary tests (include/helioselene_gb300.hpp):
g++ only, objects and programs in a temporary directory."""

import os
import shutil
import subprocess
from pathlib import Path

from conftest import ROOT

CPP = ROOT / "tests" / "cpp"
INCLUDE = ROOT / "include"
LIBDIR = ROOT / "helioselene_gb300"


def gxx() -> str:
    cxx = os.environ.get("CXX") or shutil.which("g++")
    if not cxx:
        raise RuntimeError("g++ not found")
    return cxx


def reference_root():
    """the helioselene checkout (HELIOSELENE_REF), or None where it is absent"""
    ref = Path(os.environ.get("HELIOSELENE_REF", "/root/reference"))
    return ref if (ref / "helios" / "include" / "helios.h").exists() else None


def reference_includes(ref: Path) -> list:
    return [f"-I{ref / d}" for d in ("common/include", "fp/include", "fq/include", "helios/include",
                                     "selene/include", "include")]


def build_golden_program(out_dir: Path) -> Path:
    """compile and link tests/cpp/golden_msm.cpp against libhelioselene_gb300.so"""
    exe = out_dir / "golden_msm"
    subprocess.run([gxx(), "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{INCLUDE}",
                    str(CPP / "golden_msm.cpp"), "-o", str(exe), f"-L{LIBDIR}", "-lhelioselene_gb300",
                    f"-Wl,-rpath,{LIBDIR}"], check=True, capture_output=True, text=True)
    return exe


def write_cases(golden: dict, path: Path) -> int:
    """the reference's MSM and Pedersen golden vectors in golden_msm's case format"""
    lines = []
    for curve in ("helios", "selene"):
        pt = golden[curve + "_point"]
        for v in pt["msm"]:
            lines.append(" ".join(["msm", curve, str(len(v["scalars"])), v["label"], *v["scalars"], *v["points"],
                                   v["result"]]))
        for v in pt["pedersen_commit"]:
            lines.append(" ".join(["pedersen", curve, str(len(v["values"])), v["label"], v["blinding"], v["H"],
                                   *v["values"], *v["generators"], v["result"]]))
    path.write_text("\n".join(lines) + "\n")
    return len(lines)
