"""bench.py's reference arm on the CPU: one JSON line with the keys and types
the benchmark contract fixes (impl, metric, value, unit, steps, warmup,
higher_is_better, e2e with zero transfer bytes, cpu_baseline with its kind,
cores and sample), for the planted 200 x 500 LP and the transportation LP."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _run(*args):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


@pytest.mark.parametrize("config", [0, 1])
def test_reference_arm_line(config):
    import bench
    line = _run("--config", str(config), "--steps", "3", "--warmup", "3", "--cpu-budget", "0.3")
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["steps"] == 3 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert line["unit"] == "solves/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["vs_baseline"] is None and line["data"] == "synthetic"
    assert "workload" in line["config"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["value"] == line["value"] and cb["unit"] == line["unit"] and cb["sample"]
