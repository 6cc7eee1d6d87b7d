"""The benchmark sweep harness (bkma_gb300.harness) without a GPU: its shapes
are the reference's, and its records follow google-benchmark's JSON layout
(the fields the reference's diag/utils.py reads)."""
import os
import re

import pytest

from bkma_gb300 import harness

REF = os.path.join(os.environ.get("BKMA_REFERENCE_DIR", "/root/reference"), "benchmark")


def test_records_and_aggregates():
    runs = [harness.entry("main-BKM-bench/1/1/9/128/1/1/real_time", r, 3, 10, s, 1e9, 8,
                          {"n0": 2, "n1": 3, "n2": 4, "kernel_id": 1})
            for r, s in enumerate((1.0, 2.0, 4.0))]
    assert runs[0]["real_time"] == pytest.approx(100.0)          # ms per iteration
    assert runs[0]["items_per_second"] == pytest.approx(1e10)
    assert runs[0]["bytes_per_second"] == pytest.approx(1.6e11)  # 2 x 8 B per item
    agg = {a["aggregate_name"]: a for a in harness.aggregate(runs)}
    assert set(agg) == {"mean", "median", "stddev", "cv"}
    for name, a in agg.items():
        assert a["name"].endswith("_" + name) and a["run_type"] == "aggregate"
        assert a["kernel_id"] == 1 and a["n0"] == 2
    times = [100.0, 200.0, 400.0]
    mean = sum(times) / 3
    assert agg["mean"]["real_time"] == pytest.approx(mean)
    assert agg["median"]["real_time"] == pytest.approx(200.0)
    sd = (sum((t - mean) ** 2 for t in times) / 2) ** 0.5
    assert agg["stddev"]["real_time"] == pytest.approx(sd)
    assert agg["cv"]["real_time"] == pytest.approx(sd / mean)
    assert {"date", "host_name", "num_cpus", "library_build_type"} <= set(harness.context())


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not available")
def test_shapes_are_the_references():
    src = open(os.path.join(REF, "bench_config.hpp")).read()

    def val(t):
        t = t.replace(" ", "")
        m = re.fullmatch(r"\(1<<(\d+)\)\+(\d+)", t)
        if m:
            return (1 << int(m.group(1))) + int(m.group(2))
        m = re.fullmatch(r"1<<(\d+)", t)
        return (1 << int(m.group(1))) if m else int(t)

    exps = sorted(re.findall(r"static expe e(\d)\{([^}]*)\}", src))
    assert [tuple(val(x) for x in body.split(",")) for _, body in exps] == harness.EXP_SIZES
    src = open(os.path.join(REF, "conv1d-bench.cpp")).read()
    start = src.index("configs ={")
    block = src[start:src.index("};", start)]
    confs = [tuple(int(v) for v in m.split(",")) for m in re.findall(r"\{([\d ,]+)\}", block)]
    assert confs == harness.CONV_CONFIGS
