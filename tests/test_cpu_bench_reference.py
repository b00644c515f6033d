"""bench.py's reference arm (`--impl reference`) on the host: the CPU implementation
of the path alone, timed on the same workload, metric and unit as the GPU arm.  Its
JSON line carries the keys the GPU arm's line has, a cpu_baseline describing this run
and an e2e with no host-device copies, and the process never maps the engine's
library (the arm builds its phantom with numpy and its exposures with the oracle)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUNNER = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "0"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    if e.code not in (None, 0):
        raise
with open("/proc/self/maps") as f:
    print("ENGINE_MAPPED", any("libdxmcg" in line for line in f))
"""


def test_reference_arm_line_and_no_engine():
    r = subprocess.run([sys.executable, "-c", RUNNER], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert lines[-1] == "ENGINE_MAPPED False"
    line = json.loads(next(l for l in reversed(lines) if l.startswith("{")))
    assert line["impl"] == "reference"
    assert line["unit"] == "histories/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 0
    assert line["config"]["workload"].startswith("DX on a 128x128x64 water cylinder")
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "histories/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
