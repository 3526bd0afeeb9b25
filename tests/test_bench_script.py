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


def test_host_cpu_record():
    """the e2e host record: CPU time per step and CPUs busy from two reads, with the
    cgroup and steal-time fields where the host exposes them"""
    sys.path.insert(0, str(ROOT))
    import bench
    a = bench.host_cpu_state()
    sum(i * i for i in range(200000))
    b = bench.host_cpu_state()
    d = bench.host_cpu_delta(a, b, 4)
    assert d["process_cpu_ms_per_step"] >= 0 and d["cpus_busy"] >= 0 and d["cpus_usable"] >= 1
    if "nr_throttled" in a:
        assert d["cgroup_throttled_periods"] >= 0
    if "steal_ms" in a:
        assert d["steal_ms_all_cpus"] >= 0
