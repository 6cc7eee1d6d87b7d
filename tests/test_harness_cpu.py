"""The benchmark sweep harness (bkma_gb300.harness) without a GPU: its shapes
are the reference's, and its records follow google-benchmark's JSON layout
(the fields the reference's diag/utils.py reads)."""
import os
import re

import pytest

from bkma_gb300 import harness

from oracle import reference_dir

REF = os.path.join(reference_dir() or "", "benchmark")


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


def _clean_raw_df_groups(benches):
    """The record filter and grouping of the reference's diag/utils.py
    clean_raw_df (:88-155), restated without pandas: drop _mean and
    BM_WgSize records, then read the rest three at a time as a benchmark's
    _median, _stddev and _cv, with the fields it uses."""
    rows = [b for b in benches
            if not b["name"].endswith("_mean") and not b["name"].startswith("BM_WgSize")]
    assert len(rows) % 3 == 0
    groups = [rows[i:i + 3] for i in range(0, len(rows), 3)]
    for g in groups:
        assert [r["name"].rsplit("_", 1)[1] for r in g] == ["median", "stddev", "cv"]
        assert len({r["name"].split("_")[0] for r in g}) == 1
        for r in g:
            for k in ("kernel_id", "n0", "n1", "n2", "items_per_second", "real_time", "gpu"):
                assert k in r, (r["name"], k)
    return groups


def test_aggregates_only_report_reads_like_the_reference_diag():
    benches = []
    for impl in (0, 1):
        for w in (128, 1024):
            name = f"main-BKM-bench/1/{impl}/3/{w}/1/1/real_time"
            runs = [harness.entry(name, r, 3, 10, 1.0 + r, 1e9, 4, {}) for r in range(3)]
            for r in runs:
                r.update({"gpu": 1, "n0": 8, "n1": 16, "n2": 1, "kernel_id": impl})
            benches += runs + harness.aggregate(runs)
    groups = _clean_raw_df_groups(harness.report(benches, aggregates_only=True))
    assert len(groups) == 4
    # with the per-repetition records the reference's grouping breaks: the
    # reason for --report-aggregates-only
    with pytest.raises(AssertionError):
        _clean_raw_df_groups(harness.report(benches, aggregates_only=False))


@pytest.mark.skipif(reference_dir() is None, reason="reference checkout not available")
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
