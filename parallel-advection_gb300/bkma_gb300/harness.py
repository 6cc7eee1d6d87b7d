"""Benchmark sweeps with the reference's shapes, written as google-benchmark
JSON (the format the reference's diag/utils.py reads).

Advection: the reference's EXP_SIZES e0..e9 (benchmark/bench_config.hpp:31-42)
with its physical parameters (benchmark/bench_utils.hpp:26-50: dt = 0.001,
x in [0, 1), v in [-1, 1) by line), the analytic sin(4 pi x) init and its
mean-L1 validation after the run (`err` counter), for each kernel_id and
pref_wg_size of the reference's sweep (kernel_id 0 = NDRange, 1 = AdaptiveWg;
both names select this library's in-place advection plan, whose own tile
choice ignores pref_wg_size), in FP64 (the reference's real_t) or FP32.
Conv1d: the six {batch, length, kernel, channels} configs of
benchmark/conv1d-bench.cpp:18-25 with ConvSolver semantics in FP64, constant
fills 7.3 / 1.5 / 1.0, three warm-up calls and the normalised sum of the
first length-kernel+1 values per line (`result`).

Each benchmark runs `repetitions` times; like google-benchmark with
--benchmark_repetitions it reports every repetition and the _mean, _median,
_stddev and _cv aggregates, with items_per_second = cells per second and
bytes_per_second = 2 x element size x cells per second. With
--report-aggregates-only it writes the aggregates alone, as the reference's
diag/launch_benchmarks.sh runs its benchmarks: the input diag/utils.py reads.

  python -m bkma_gb300.harness [--out sweep.json] [--dtype f64|f32]
                               [--repetitions 3] [--only adv|conv] [--sizes 0,5,9]
                               [--conv-configs 0,3] [--max-cells N]
                               [--report-aggregates-only]

--max-cells caps an advection shape's n0 so that n0 x n1 x n2 <= N (the
record keeps the reference's n0 as n0_full); --conv-configs picks conv
configs by index.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import platform
import statistics
import time

# (n0, n1, n2) of the reference's EXP_SIZES, in order e0..e9
EXP_SIZES = [
    (1 << 17, 1 << 14, 1),
    (1 << 10, 1 << 11, 1 << 10),
    (1 << 10, 1 << 14, 1 << 7),
    (1 << 27, 1 << 4, 1),
    (1 << 20, 1 << 4, 1 << 7),
    (1 << 21, 1 << 10, 1),
    (1 << 14, 1 << 10, 1 << 7),
    (1, 1 << 10, (1 << 6) + 1),
    (1, 1 << 10, 1 << 21),
    (1 << 11, 1 << 10, 1 << 10),
]
# {batch_size, input_length, kernel_size, channels}
CONV_CONFIGS = [
    (16384, 512, 3, 1),
    (1024, 512, 3, 1),
    (32768, 128, 3, 9),
    (16384, 256, 5, 6),
    (16384, 512, 5, 3),
    (16384, 1024, 11, 1),
]
ADV_IMPLS = (0, 1)  # kernel_id: 0 = NDRange, 1 = AdaptiveWg
ADV_PREF_WG = (128, 1024)
PERF_KEYS = ("real_time", "cpu_time", "items_per_second", "bytes_per_second")


def aggregate(runs: list[dict]) -> list[dict]:
    """google-benchmark repetition aggregates of `runs` (one benchmark):
    _mean, _median, _stddev and _cv records carrying the runs' counters."""
    out = []
    base = runs[0]
    for agg in ("mean", "median", "stddev", "cv"):
        e = dict(base)
        e["name"] = f"{base['run_name']}_{agg}"
        e["run_type"] = "aggregate"
        e["aggregate_name"] = agg
        e["repetitions"] = len(runs)
        for k in PERF_KEYS:
            vals = [r[k] for r in runs]
            mean = statistics.fmean(vals)
            sd = statistics.stdev(vals) if len(vals) > 1 else 0.0
            e[k] = {"mean": mean, "median": statistics.median(vals), "stddev": sd,
                    "cv": (sd / mean if mean else 0.0)}[agg]
        if agg == "cv":
            e["aggregate_unit"] = "percentage"
        out.append(e)
    return out


def report(benches: list[dict], aggregates_only: bool) -> list[dict]:
    """The records written out: all of them, or only the aggregates, as
    google-benchmark's --benchmark_report_aggregates_only=true (which
    diag/launch_benchmarks.sh:61 passes) writes them. diag/utils.py:88-155
    (clean_raw_df) reads that form: it drops the _mean records and takes the
    rest as (_median, _stddev, _cv) triples of one benchmark."""
    if not aggregates_only:
        return benches
    return [b for b in benches if b.get("run_type") == "aggregate"]


def entry(run_name: str, rep: int, reps: int, iterations: int, seconds: float, items: float,
          elem_bytes: int, counters: dict) -> dict:
    """One google-benchmark iteration record (UseRealTime, unit ms)."""
    ms = seconds / iterations * 1e3
    e = {"name": run_name, "family_index": 0, "per_family_instance_index": 0,
         "run_name": run_name, "run_type": "iteration", "repetitions": reps,
         "repetition_index": rep, "threads": 1, "iterations": iterations,
         "real_time": ms, "cpu_time": ms, "time_unit": "ms",
         "items_per_second": items * iterations / seconds,
         "bytes_per_second": items * iterations * elem_bytes * 2 / seconds}
    e.update(counters)
    return e


def context() -> dict:
    return {"date": datetime.datetime.now().isoformat(timespec="seconds"),
            "host_name": platform.node(), "executable": "bkma_gb300.harness",
            "num_cpus": os.cpu_count() or 1, "mhz_per_cpu": 0, "cpu_scaling_enabled": False,
            "caches": [], "load_avg": [], "library_build_type": "release"}


def _timed(fn, min_seconds: float, max_iters: int) -> tuple[int, float]:
    """Run fn (one iteration each) until min_seconds of device time have
    passed, at least once; CUDA events on the current stream."""
    import torch
    iters, total = 0, 0.0
    while iters < max_iters and (iters == 0 or total < min_seconds):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        total += a.elapsed_time(b) / 1e3
        iters += 1
    return iters, total


def advection_sweep(bkma, dev, dtype: str, reps: int, min_seconds: float,
                    sizes=None, max_cells: int | None = None) -> list[dict]:
    import torch
    tdt = torch.float64 if dtype == "f64" else torch.float32
    es = 8 if dtype == "f64" else 4
    out = []
    for idx, (n0_full, n1, n2) in enumerate(EXP_SIZES):
        if sizes is not None and idx not in sizes:
            continue
        n0 = n0_full if max_cells is None else max(1, min(n0_full, max_cells // (n1 * n2)))
        t0 = time.perf_counter()
        plan = bkma.AdvectionPlan(n0, n1, n2, dtype=dtype, dt=0.001, minX=0.0, maxX=1.0,
                                  minVx=-1.0, maxVx=1.0)
        plan_s = time.perf_counter() - t0
        data = torch.empty((n0, n1, n2), dtype=tdt, device=dev)
        cells = n0 * n1 * n2
        info = plan.info()
        for impl in ADV_IMPLS:
            for w in ADV_PREF_WG:
                plan.fill(data, mode=0)
                steps = 0
                runs = []
                name = f"main-BKM-bench/1/{impl}/{idx}/{w}/1/1/real_time"
                for rep in range(reps):
                    iters, secs = _timed(lambda: plan.step(data), min_seconds, 1000)
                    steps += iters
                    runs.append(entry(name, rep, reps, iters, secs, cells, es, {}))
                plan.status()
                err, _ = plan.validate(data, steps)
                for r in runs:
                    r.update({"gpu": 1, "n0": n0, "n1": n1, "n2": n2, "n0_full": n0_full,
                              "kernel_id": impl,
                              "pref_wg_size": w, "seq_size0": 1, "seq_size2": 1, "err": err,
                              "dtype": dtype, "path": info["path"],
                              "exception_lines": info["exception_lines"],
                              "plan_seconds": plan_s})
                out.extend(runs)
                out.extend(aggregate(runs))
        del data, plan
        torch.cuda.empty_cache()
    return out


def conv_sweep(bkma, dev, reps: int, configs=None) -> list[dict]:
    """ConvSolver semantics, FP64 (the reference's real_t)."""
    import torch
    tdt = torch.float64
    out = []
    for idx, (batch, length, k, ch) in enumerate(CONV_CONFIGS):
        if configs is not None and idx not in configs:
            continue
        n0, n1, n2 = batch, length * ch, 1
        plan = bkma.Conv1dPlan(n0, ch, ch, length, k, dtype="f64", semantics="reference",
                               n2=n2)
        weight = torch.full((k, ch, ch), 1.5, dtype=tdt, device=dev)
        bias = torch.full((ch,), 1.0, dtype=tdt, device=dev)
        warm = torch.full((n0, n1, n2), 7.3, dtype=tdt, device=dev)
        for _ in range(3):  # warm-up calls, as the reference
            plan.run(warm, weight, bias)
        del warm
        data = torch.empty((n0, n1, n2), dtype=tdt, device=dev)
        runs = []
        name = f"main-BKM-bench/{idx}/iterations:1/real_time"
        result = None
        nw = length - k + 1  # the reference normalises the first L-K+1 values
        for rep in range(reps):
            data.fill_(7.3)
            torch.cuda.synchronize()
            iters, secs = _timed(lambda: plan.run(data, weight, bias), 0.0, 1)
            result = float(data[:, :nw, :].sum().item() / (n0 * nw * n2))
            runs.append(entry(name, rep, reps, iters, secs, n0 * n1 * n2, 8, {}))
        plan.status()
        for r in runs:
            r.update({"n0": n0, "n1": n1, "n2": n2, "pref_wg_size": 512, "seq_size0": 1,
                      "seq_size2": 1, "batch_size": batch, "input_length": length,
                      "kernel_size": k, "channels": ch, "result": result, "dtype": "f64"})
        out.extend(runs)
        out.extend(aggregate(runs))
        del data, plan, weight, bias
        torch.cuda.empty_cache()
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="bkma_sweep.json")
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"],
                    help="advection storage; f64 = the reference's real_t")
    ap.add_argument("--repetitions", type=int, default=3)
    ap.add_argument("--min-seconds", type=float, default=0.2,
                    help="device time per advection repetition")
    ap.add_argument("--only", choices=["adv", "conv"], default=None)
    ap.add_argument("--sizes", default=None, help="comma list of EXP_SIZES indices")
    ap.add_argument("--conv-configs", default=None, help="comma list of conv config indices")
    ap.add_argument("--max-cells", type=int, default=None,
                    help="cap n0 of an advection shape so that it has at most this many cells")
    ap.add_argument("--report-aggregates-only", action="store_true",
                    help="write only the aggregate records (google-benchmark's "
                         "--benchmark_report_aggregates_only; the input of diag/utils.py)")
    a = ap.parse_args(argv)
    import torch

    import bkma_gb300 as bkma
    dev = torch.device("cuda", 0)
    sizes = None if a.sizes is None else {int(s) for s in a.sizes.split(",")}
    confs = None if a.conv_configs is None else {int(s) for s in a.conv_configs.split(",")}
    benches = []
    t0 = time.perf_counter()
    if a.only in (None, "adv"):
        benches += advection_sweep(bkma, dev, a.dtype, a.repetitions, a.min_seconds, sizes,
                                   a.max_cells)
    if a.only in (None, "conv"):
        benches += conv_sweep(bkma, dev, a.repetitions, confs)
    doc = {"context": context(), "benchmarks": report(benches, a.report_aggregates_only)}
    doc["context"]["wall_seconds"] = round(time.perf_counter() - t0, 3)
    with open(a.out, "w") as f:
        json.dump(doc, f, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
