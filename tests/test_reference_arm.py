"""bench.py --impl reference (the reference arm) on the host: one JSON line with the GPU arm's
metric, unit and configuration, the contract's cpu_baseline and e2e keys, and no trace of this
package or its CUDA library in the process (the arm times the oracle port alone)."""
import ast
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_PROBE = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3", "--ref-solves", "500"]
runpy.run_path("bench.py", run_name="__main__")
mods = sorted(m for m in sys.modules if m.startswith("traditional_dic_gb300") or m == "__graft_entry__")
maps = open("/proc/self/maps").read()
print("PROBE " + repr((mods, "libtdic_gb300" in maps)))
"""


def test_reference_arm_line_and_isolation(oracle):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-c", _PROBE], cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT and line["higher_is_better"] is True
    assert line["config"] == bench.run_config(2048, "dataflow")
    assert line["steps"] == 1 and line["warmup"] == 3 and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    probe = [ln for ln in r.stdout.splitlines() if ln.startswith("PROBE ")]
    mods, lib_loaded = ast.literal_eval(probe[0][len("PROBE "):])
    assert mods == [] and not lib_loaded
