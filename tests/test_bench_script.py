"""bench.py, __graft_entry__.py and the batched-form runner compile, and bench.py parses
its flags, without a GPU."""

import pathlib
import py_compile
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_scripts_compile(tmp_path):
    for name in ("bench.py", "__graft_entry__.py", "helioselene_gb300/batchrun.py"):
        py_compile.compile(str(ROOT / name), cfile=str(tmp_path / (name.replace("/", "_") + "c")), doraise=True)


def test_bench_help():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--ba-rounds"):
        assert flag in r.stdout
