"""The reference arm of bench.py (`--impl reference`) on the CPU, at 32^3
(SARAS_BENCH_N): one JSON line with the benchmark's metric and the keys the
arm promises (its own cpu_baseline and an e2e of zero copies), timed steps
that are full solves to the tolerance, and no product library in the
process: the arm times the oracle alone."""
import json
import os
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[1]

CHILD = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    if e.code not in (None, 0):
        raise
maps = open("/proc/self/maps").read()
print("LOADED", json.dumps({"product": "libsaras_gb300" in maps, "oracle": "liboracle" in maps}))
"""


def test_reference_arm_line():
    env = dict(os.environ, SARAS_BENCH_N="32")
    r = subprocess.run([sys.executable, "-c", "import json\n" + CHILD], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("256^3 MG solve time") and d["unit"] == "ms"
    assert d["higher_is_better"] is False and d["n_gpus"] == 1
    assert d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    assert d["config"]["n"] == 32 and "Poisson 32^3" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # timed steps are full solves to the tolerance
    assert d["full_solve_cycles"] > 5
    loaded = json.loads(r.stdout.split("LOADED", 1)[1].strip().splitlines()[0])
    assert loaded == {"product": False, "oracle": True}, loaded
