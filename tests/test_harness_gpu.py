"""The benchmark sweep harness on the GPU, run as a user runs it
(python -m bkma_gb300.harness), on a reduced list: EXP_SIZES e7 (1 x 1024 x
65) and e5 (lines of 1024 contiguous cells, n0 capped to 16384 lines), FP64
(the reference's real_t), and conv config 1 of benchmark/conv1d-bench.cpp:18-25
({1024, 512, 3, 1}, ConvSolver semantics). Its aggregates-only JSON must read
like google-benchmark's in the reference's diag/utils.py:73-158 (records
grouped as _median/_stddev/_cv triples with the fields it uses), the rates
must be positive, the advection shapes must pass the reference's own check
(mean L1 against sin(4 pi (x - v t)) below 1e-6, tests/validation_unittests.cpp)
and the conv result must be the constant-fill value bias + C K 1.5 x 7.3
(src/tools/validation.hpp:84-156)."""
import json
import os
import subprocess
import sys

import pytest

from test_harness_cpu import _clean_raw_df_groups

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_harness_sweep_json(bkma, cuda, tmp_path):
    out = tmp_path / "sweep.json"
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join(
        [os.path.join(ROOT, "parallel-advection_gb300"), env.get("PYTHONPATH", "")])
    cmd = [sys.executable, "-m", "bkma_gb300.harness", "--out", str(out), "--dtype", "f64",
           "--repetitions", "2", "--min-seconds", "0.02", "--sizes", "5,7",
           "--max-cells", str(1 << 24), "--conv-configs", "1", "--report-aggregates-only"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    doc = json.loads(out.read_text())
    assert {"date", "host_name", "num_cpus"} <= set(doc["context"])
    benches = doc["benchmarks"]
    assert all(b["run_type"] == "aggregate" for b in benches)
    adv = [b for b in benches if "n0_full" in b]
    conv = [b for b in benches if "kernel_size" in b]
    # 2 shapes x 2 kernel ids x 2 work-group sizes, 4 aggregates each; 1 conv config
    assert len(adv) == 2 * 2 * 2 * 4 and len(conv) == 4
    groups = _clean_raw_df_groups(adv)
    assert len(groups) == 8
    for b in adv:
        if b["aggregate_name"] in ("mean", "median"):
            assert b["items_per_second"] > 0 and b["real_time"] > 0
        assert b["err"] < 1e-6, (b["name"], b["err"])
        assert b["dtype"] == "f64"
    assert {(b["n0"], b["n1"], b["n2"]) for b in adv} == {(1, 1024, 65), (16384, 1024, 1)}
    for b in conv:
        assert b["batch_size"] == 1024 and b["kernel_size"] == 3 and b["channels"] == 1
        want = 1.0 + b["channels"] * b["kernel_size"] * 1.5 * 7.3
        assert abs(b["result"] - want) <= 1e-9 * want, b["result"]
        if b["aggregate_name"] == "median":
            assert b["items_per_second"] > 0
