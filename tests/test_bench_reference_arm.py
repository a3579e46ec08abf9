"""bench.py --impl reference: the reference's CPU loop for the SpMV workload,
timed on the host cores, printing the same JSON line as the GPU arm (with
impl, cpu_baseline and a zero-copy e2e).  Runs without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "65536",
                          "--steps", "2", "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] >= 3 and d["n_gpus"] == 1
    assert d["config"]["n"] == 65536 and d["config"]["nnz"] > 65536
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_loads_no_library_code():
    """The reference arm must time the reference's loop with nothing of this
    library in the process: no libtbsla_gb300.so mapped after a run."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--n', '20000', '--steps', '1', "
            "'--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED' if 'libtbsla_gb300' in maps or 'libtbsla.so' in maps else 'CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "CLEAN"


def test_clock_sampler_waits_for_its_first_sample(tmp_path, monkeypatch):
    """The clock sampler starts nvidia-smi before a timed region and returns
    only once the first sample is in (the tool's start-up slowed host copies
    beside it), then parses clocks and throttle reasons; a tool that exits
    at once does not hold the caller.  A fake nvidia-smi on PATH, no GPU."""
    import importlib.util
    import time

    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\nsleep 0.4\n"
                    "while true; do echo '2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Active'; "
                    "sleep 0.05; done\n")
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    c = bench.Clocks(0)
    t0 = time.time()
    c.start()
    assert time.time() - t0 >= 0.35 and c.lines
    d = c.stop()
    assert d["sm_mhz"] == 2070.0 and d["sm_max_mhz"] == 2070.0 and d["reasons"] == ["sw_power_cap"]
    assert d["samples"] >= 1
    fake.write_text("#!/bin/sh\nexit 0\n")
    c = bench.Clocks(0)
    t0 = time.time()
    c.start()
    assert time.time() - t0 < 2.0
    assert c.stop()["samples"] == 0
