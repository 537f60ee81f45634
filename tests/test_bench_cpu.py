"""bench.py's reference arm (the CPU implementation of the path, no GPU) keeps
the one-JSON-line contract: the metric, unit and config of our own arm, impl
"reference", a cpu_baseline describing the run and an e2e object with zero
host-device bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "small",
                        "--steps", "1", "--warmup", "1", "--cpu-seconds", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config"):
        assert k in line, k
    assert line["impl"] == "reference" and line["unit"] == "reflections/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1
    assert line["config"]["workload"].startswith("96^3") or "96" in line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "reflections/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
