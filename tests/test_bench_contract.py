"""bench.py's JSON line for the arms that run without a GPU: the readout
workload's reference arm (the oracle's serial FIFO, the reference's
src/event_readout.cpp restated) and a reference arm with no counterpart in the
reference (serving), which prints its `unavailable` line and exits 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench_line(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_readout_reference_arm_line():
    d = bench_line("--impl", "reference", "--workload", "readout", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["unit"] == "events/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0 and d["data"] == "synthetic"
    assert d["config"]["workload"] == "readout" and d["config"]["events_per_batch"] == 1 << 22
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_without_counterpart_is_unavailable():
    d = bench_line("--impl", "reference", "--workload", "serving")
    assert d["impl"] == "reference" and d["unavailable"]
