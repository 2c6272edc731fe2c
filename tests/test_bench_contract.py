"""bench.py's reference arm on the CPU: one JSON line with the keys the
benchmark contract names (impl, metric, value, e2e with zero copy bytes,
cpu_baseline describing the run)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


# runs the reference arm in-process, then reports which native libraries that
# process mapped: the arm must not load the GPU library
RUNNER = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED", int("libturner_gb300" in maps), int("liboracle" in maps))
"""


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "-c", RUNNER], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    assert "MAPPED 0 1" in r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Mrays/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["e2e"] == {"value": d["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and "rows" in cb["sample"]
    assert d["config"]["workload"].startswith("sphere_room_327k_1920x1080_16spp_d3")
