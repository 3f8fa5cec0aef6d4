"""The reference arm of bench.py (the oracle's OpenMP loops on the host
cores; no GPU) prints one JSON line with the keys its consumers read: the
metric and unit of the GPU arm, the CPU baseline that describes the run, and
an end-to-end entry with no host-device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                         check=True, capture_output=True, text=True, cwd=ROOT, timeout=600)
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference"
    assert d["metric"] == "bond-updates/s" and d["unit"] == "bond-updates/s"
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "crack_branching_2d_pmb_verlet"
    assert d["config"]["nodes"] == 1_600_000 and d["config"]["bonds"] == 44_699_236
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_without_a_counterpart_says_so():
    d = _run("--workload", "warm_start", "--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference" and d["unavailable"]
