"""bench.py's GPU arm (quick mode: the headline advection run only): one JSON
line with the metric, the roofline of the timed kernel, clock samples and
the launch count."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_quick_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--quick", "--steps", "5", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "roofline", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["value"] > 0 and d["steps"] == 5 and d["n_gpus"] == 1
    assert d["gpu_launches"] >= d["steps"]
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s"
    assert 0.0 < rf["frac"] < 1.2 and rf["peak"] > 0
    assert abs(rf["achieved"] / rf["peak"] - rf["frac"]) < 1e-9
    assert "workload" in d["config"]
    if d["clocks"] is not None:
        assert d["clocks"]["samples"] >= 1 and d["clocks"]["sm_mhz"] > 0
