"""bench.py's command line and its reference arm, which runs on the host cores only: the JSON
line it prints carries the keys of the benchmark contract (a 16^3-cell workload keeps it short)."""
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_command_line_has_the_contract_flags():
    out = subprocess.run([sys.executable, "bench.py", "--help"], cwd=ROOT, capture_output=True, text=True,
                         check=True, timeout=120).stdout
    for flag in ("--gpus", "--steps", "--warmup", "--impl"):
        assert flag in out


def test_reference_arm_line():
    t0 = time.perf_counter()
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--cells", "16", "--steps", "2",
                        "--warmup", "1", "--ref-sample-iters", "2"], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    wall = time.perf_counter() - t0
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 2
    # a step's time is the time the step took (the bounded sample), so the timed steps fit the run
    assert line["steps"] * line["ms_per_step"] / 1e3 <= wall
    assert line["solve_seconds_extrapolated"] > 0
    assert line["config"]["workload"].startswith("polycrystal 2-level AMR: 16^3 cells")
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
