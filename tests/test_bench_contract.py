"""The benchmark's JSON line (reference arm, runnable on the CPU): one line
with the keys and types the measurement contract names."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
  cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
         "si2_fcc_48", "--steps", "1", "--warmup", "0", "--cpu-sample-kpts", "1"]
  r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
  assert r.returncode == 0, r.stderr[-2000:]
  lines = [l for l in r.stdout.splitlines() if l.strip()]
  assert len(lines) == 1
  d = json.loads(lines[0])
  assert d["impl"] == "reference"
  for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
            "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
            "cpu_baseline", "e2e"):
    assert k in d, k
  assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
  assert d["config"]["workload"] == "si2_fcc_48"
  cb = d["cpu_baseline"]
  assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
  assert "1 of 8 k-points" in cb["sample"]
  e = d["e2e"]
  assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
