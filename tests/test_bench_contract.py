"""CPU test of bench.py's reference arm: it runs on the host cores only, prints
one JSON line whose metric, unit, direction and workload are the GB300 arm's,
with a cpu_baseline and a zero-copy e2e, and ranks other than 0 print nothing."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CMD = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--config", "small",
       "--steps", "1", "--warmup", "3", "--cpu-seconds", "1"]


def _run(env_extra=None):
    env = dict(os.environ, **(env_extra or {}))
    res = subprocess.run(CMD, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    return [ln for ln in res.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_line(lib, port):
    import bench
    import simplemoc_gb300 as sm
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC
    assert d["unit"] == "integrations/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == bench._workload("small", sm.CONFIGS["small"])
    assert d["steps"] == 1 and d["warmup"] == 3 and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    # timed with the reference's own timing flags (src/Makefile:77), stated in the line
    assert "-Ofast" in d["config"]["compiler_flags"] and "-fopenmp" in cb["compiler_flags"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly(lib, port):
    assert _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"}) == []


def test_flux_error_figures():
    """bench.flux_errors: normwise, per FSR (max norm over its groups) and per
    element, on a case with known answers."""
    import numpy as np

    import bench
    ref = np.array([1.0, 2.0, 4.0, 8.0, 1.0, 1.0])        # two FSRs of three groups
    a = ref.copy()
    a[1] += 1e-3                                          # FSR 0: 1e-3 / 4
    a[4] += 2e-3                                          # FSR 1: 2e-3 / 8
    e = bench.flux_errors(a, ref, 3)
    assert abs(e["normwise"] - 2e-3 / 8) < 1e-15
    assert abs(e["per_fsr_max"] - 2.5e-4) < 1e-15
    assert abs(e["per_element_max"] - 2e-3) < 1e-15
    assert e["per_fsr_frac_within_contract"] == 0.0
