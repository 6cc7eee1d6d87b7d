#!/usr/bin/env python
"""Benchmark of the BKMA hot path on GB300.

Workload (default, one GPU): large single advection — FP32 field
n0=2048 x n1=1024 x n2=512 (2^30 cells, 4 GiB), degree-5 reference stencil,
line velocities v_i = -1 + 2 i/(n0-1), dx = 1/1024, dt = 0.001, init
sin(2 pi x) + U[-0.01, 0.01] (seeded, generated on the device), 50 time steps.
A bench "step" is one time step over the whole field (one kernel launch).
The field is 4 GiB, far larger than L2 (129 MB), so no flush is needed.

Prints ONE JSON line. Reference arm (--impl reference): the CPU oracle port of
the reference's AdvectionSolver + AdaptiveWg schedule, FP64, all host cores,
on a bounded sample of the same workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "parallel-advection_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N0, N1, N2 = 2048, 1024, 512  # --n0/--n1/--n2 change the field for profiling captures only
DT, MINX, MAXX = 0.001, 0.0, 1.0
NOISE, SEED = 0.01, 12345
CFG_STEPS = 50
METRIC = "advection GCells/s (FP32 storage, FP64 foot-point, degree 5)"
UNIT = "GCells/s"
WORKLOAD = "large single advection FP32 2048x1024x512, degree 5, 50 steps"
# per plan path: the ncu DRAM traffic (bytes per launch on the bench field) of
# the kernel that path launches; only the TMA path (the bench field's) is captured
PROFILE_JSON = {1: os.path.join(ROOT, "profiles", "adv_tma_f32_2048x1024x512.json")}


def velocities(n0: int):
    """v_i = -1 + 2 i / (n0 - 1); a single line (profiling shapes) moves at -1."""
    import numpy as np
    return -1.0 + 2.0 * np.arange(n0, dtype=np.float64) / max(n0 - 1, 1)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """SM clock, power and clock-event reasons sampled during the timed
    region: NVML (the NVIDIA driver's libnvidia-ml, read-only queries) every 5 ms
    from a thread, the GPU matched by UUID; nvidia-smi every 200 ms when NVML
    cannot be loaded."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.nv = None
        self.samples = []
        self.running = False

    def _nvml_handle(self):
        import ctypes as C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = C.c_void_p()
        uuid = None
        try:
            import torch
            u = getattr(torch.cuda.get_device_properties(self.index), "uuid", None)
            if u is not None:
                uuid = "GPU-" + str(u) if not str(u).startswith("GPU-") else str(u)
        except Exception:
            uuid = None
        ok = uuid is not None and lib.nvmlDeviceGetHandleByUUID(uuid.encode(), C.byref(h)) == 0
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
            return None
        return lib, h

    def _poll(self):
        import ctypes as C
        lib, h = self.nv
        sm, mx, pw, rs = C.c_uint(), C.c_uint(), C.c_uint(), C.c_ulonglong()
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx))
        while self.running:
            if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(sm)) == 0 and \
                    get_reasons(h, C.byref(rs)) == 0:
                lib.nvmlDeviceGetPowerUsage(h, C.byref(pw))
                self.samples.append((sm.value, mx.value, pw.value / 1000.0, rs.value))
            time.sleep(0.005)

    def start(self):
        try:
            self.nv = self._nvml_handle()
        except Exception:
            self.nv = None
        if self.nv is not None:
            self.running = True
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.nv is not None:
            self.running = False
            self.t.join(timeout=1)
            if not self.samples:
                return None
            reasons = set()
            for _, _, _, r in self.samples:
                for bit, name in self.REASONS.items():
                    if r & bit:
                        reasons.add(name)
            return {"sm_mhz": statistics.median(x[0] for x in self.samples),
                    "sm_max_mhz": max(x[1] for x in self.samples),
                    "power_w": statistics.median(x[2] for x in self.samples),
                    "samples": len(self.samples), "source": "nvml, 5 ms",
                    "reasons": sorted(reasons)}
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r.split(", ") for r in self.lines if r]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "source": "nvidia-smi, 200 ms", "reasons": sorted(reasons)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# --------------------------------------------------------------- reference arm
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    from oracle import AdvParams, Oracle
    orc = Oracle()
    cores = os.cpu_count() or 1
    # bounded sample: S whole slabs (all n1 x n2 cells of S velocity lines)
    p = AdvParams(n0=N0, n1=N1, n2=N2, dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0)
    vel = velocities(N0)
    S = 4
    rng = np.random.default_rng(SEED)
    x = np.arange(N1) / N1
    f = np.ascontiguousarray(np.sin(2 * np.pi * x)[None, :, None] +
                             NOISE * rng.uniform(-1, 1, (S, N1, N2)))
    t0 = time.perf_counter()
    orc.adv_step(p, f, 1, velocity=vel[:S], nthreads=cores)
    one = time.perf_counter() - t0
    # size the sample so one step takes about 1-3 s
    S = int(max(1, min(N0, S * max(1.0, 1.5 / max(one, 1e-3)))))
    f = np.ascontiguousarray(np.sin(2 * np.pi * x)[None, :, None] +
                             NOISE * rng.uniform(-1, 1, (S, N1, N2)))
    for _ in range(args.warmup):
        orc.adv_step(p, f, 1, velocity=vel[:S], nthreads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.adv_step(p, f, 1, velocity=vel[:S], nthreads=cores)
    el = time.perf_counter() - t0
    cells = S * N1 * N2 * args.steps
    v = cells / el / 1e9
    sample = f"{S} of {N0} velocity slabs ({S}x{N1}x{N2} FP64 cells) per step"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": sample, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def cpu_baseline_sample(cores: int):
    """The oracle (C restatement of AdvectionSolver + AdaptiveWg, FP64) on a
    bounded sample of the workload: about 10-20 s of host work."""
    import numpy as np
    from oracle import AdvParams, Oracle
    orc = Oracle()
    p = AdvParams(n0=N0, n1=N1, n2=N2, dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0)
    vel = velocities(N0)
    x = np.arange(N1) / N1
    rng = np.random.default_rng(SEED)
    S = 2
    f = np.ascontiguousarray(np.sin(2 * np.pi * x)[None, :, None] +
                             NOISE * rng.uniform(-1, 1, (S, N1, N2)))
    t0 = time.perf_counter()
    orc.adv_step(p, f, 1, velocity=vel[:S], nthreads=cores)
    one = time.perf_counter() - t0
    S = int(max(1, min(N0, S * 3.0 / max(one, 1e-3))))
    f = np.ascontiguousarray(np.sin(2 * np.pi * x)[None, :, None] +
                             NOISE * rng.uniform(-1, 1, (S, N1, N2)))
    steps = 6
    t0 = time.perf_counter()
    orc.adv_step(p, f, steps, velocity=vel[:S], nthreads=cores)
    el = time.perf_counter() - t0
    return {"value": S * N1 * N2 * steps / el / 1e9, "unit": UNIT, "cores": cores,
            "kind": "port",
            "sample": f"{steps} steps over {S} of {N0} velocity slabs ({S}x{N1}x{N2} FP64 cells), "
                      f"{el:.1f} s"}


def cpu_conv_sample(cores: int, C: int = 128, L: int = 8192, K: int = 7):
    """conv1d on the host cores, FP64, on a bounded sample of the conv
    workload: the oracle's torch-semantics form (cross-correlation, the op the
    GPU path computes) on S batch items, and the reference's ConvSolver
    semantics (the reference's own conv1d operator, src/solvers/ConvSolver.hpp:20-44:
    the same Cin*K multiply-adds per output) on S lines of C*L packed values.
    TFLOP/s counts 2*Cout*Cin*K*(L-K+1) per item for both."""
    import numpy as np
    from oracle import Oracle
    orc = Oracle()
    S = 4 * max(1, cores)
    rng = np.random.default_rng(SEED)
    s = 1.0 / (C * K) ** 0.5
    x = rng.uniform(-1, 1, (S, C, L)) * s
    w = rng.uniform(-1, 1, (C, C, K)) * s
    flops = 2.0 * S * C * C * K * (L - K + 1)
    t0 = time.perf_counter()
    orc.conv_torch(x, w, np.zeros(C), nthreads=cores)
    el = time.perf_counter() - t0
    data = np.ascontiguousarray(rng.uniform(-1, 1, (S, C * L, 1)) * s)
    wr = np.ascontiguousarray(np.transpose(w, (2, 1, 0)))  # (K, Cin, Cout)
    t0 = time.perf_counter()
    orc.conv_ref_step(data, wr, np.zeros(C), K, C, L, nthreads=cores)
    el_ref = time.perf_counter() - t0
    return {"value": flops / el / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
            "sample": f"{S} of 256 batch items (C={C}, L={L}, K={K}), FP64, {el:.1f} s",
            "convsolver_semantics_tflops": flops / el_ref / 1e12,
            "convsolver_semantics_sample": f"{S} lines of {C}x{L} packed values, FP64, "
                                           f"{el_ref:.1f} s"}


def cpu_adv_fields_sample(fields, cores: int, slabs: int, steps: int):
    """The oracle (AdvectionSolver + AdaptiveWg restated, FP64) over the first
    `slabs` velocity slabs of every field in `fields` (dicts with n0, n1, n2,
    degree, ref, velocity, dt), `steps` steps each; GCells/s over the sample."""
    import numpy as np
    from oracle import AdvParams, Oracle
    orc = Oracle()
    cells, el = 0, 0.0
    for f in fields:
        n0, n1, n2 = f["n0"], f["n1"], f["n2"]
        S = min(n0, slabs)
        p = AdvParams(n0=n0, n1=n1, n2=n2, dt=f["dt"], minX=MINX, maxX=MAXX,
                      minVx=f.get("minVx", -1.0), maxVx=f.get("maxVx", 1.0))
        x = np.arange(n1) / n1
        d = np.ascontiguousarray(np.broadcast_to(np.sin(2 * np.pi * x)[None, :, None],
                                                 (S, n1, n2)))
        t0 = time.perf_counter()
        orc.adv_step(p, d, steps, velocity=np.asarray(f["velocity"][:S]), degree=f["degree"],
                     ref_weights=f["ref"], nthreads=cores)
        el += time.perf_counter() - t0
        cells += S * n1 * n2 * steps
    return cells / el / 1e9, cells, el


def config1_block(bkma_gb300, dev, cores: int):
    """The CPU-runnable advection workload as stated: FP64 512 x 1024 x 1,
    v_i = -1 + 2 i / 511 (velocity array), dx = 1/1024, dt = 0.001, degree 5,
    sin(2 pi x) + U[-0.01, 0.01] from numpy's default_rng(12345), 10 steps.
    It is L2-resident (4 MiB): a parity workload, not a roofline one. Reports
    the plain FP64 kernel (the reference's per-cell math), the staged FP64
    kernel (FP64 arithmetic), the FP64 default (contiguous lines in FP32-pair
    arithmetic), the FP32 kernels, and the 10 steps fused in one launch for
    each arithmetic (GCells/s over 10-step runs, median of 5), their error
    against the plain form after the 10 steps, and the oracle on the host
    cores on the whole workload."""
    import numpy as np
    import torch
    n0, n1, n2, steps = 512, 1024, 1, 10
    out = {"workload": "plain advection FP64 512x1024x1, v_i = -1 + 2i/511, dt = 0.001, "
                       "degree 5, sin(2 pi x) + U[-0.01, 0.01] (seed 12345), 10 steps",
           "unit": "GCells/s", "l2": "L2-resident (4 MiB field)"}
    try:
        vel = -1.0 + 2.0 * np.arange(n0) / (n0 - 1)
        rng = np.random.default_rng(SEED)
        x = np.arange(n1) / n1
        f0 = np.ascontiguousarray(np.sin(2 * np.pi * x)[None, :, None]
                                  + NOISE * rng.uniform(-1, 1, (n0, n1, n2)))
        kw = dict(dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0, velocity=vel)
        staged = bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f64", **kw)
        staged.set_tile(1, 5, 256, 0)  # FP64 arithmetic, the staged kernel's own default tile
        plans = {"plain_fp64": (bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f64", impl="plain",
                                                         **kw), torch.float64),
                 "staged_fp64": (staged, torch.float64),
                 "pair_fp64": (bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f64", **kw),
                               torch.float64),
                 "fp32": (bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f32", **kw),
                          torch.float32)}
        # the 10 steps in one launch, each line held in shared memory: the
        # same bits as one step per launch (FP64 staged arithmetic, FP32-pair
        # arithmetic of the FP64 default, FP32)
        for name, tdt, dt_name in (("staged_fp64_fused", torch.float64, "f64"),
                                   ("pair_fp64_fused", torch.float64, "f64"),
                                   ("fp32_fused", torch.float32, "f32")):
            pl = bkma_gb300.AdvectionPlan(n0, n1, n2, dtype=dt_name, **kw)
            if name == "staged_fp64_fused":
                pl.set_tile(1, 5, 256, 0)
            pl.set_fusion(steps)
            plans[name] = (pl, tdt)
        st = torch.cuda.current_stream()
        res = {}
        for name, (pl, tdt) in plans.items():
            d = torch.tensor(f0, dtype=tdt, device=dev)
            pl.step(d, nsteps=steps)
            times = []
            for _ in range(5):
                d.copy_(torch.tensor(f0, dtype=tdt, device=dev))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                pl.step(d, nsteps=steps)
                b.record(st)
                torch.cuda.synchronize()
                times.append(a.elapsed_time(b))
            pl.status()
            res[name] = d
            out[name] = {"gcells_s": n0 * n1 * n2 * steps / (statistics.median(times) / 1e3) / 1e9}
        ref = res["plain_fp64"]
        for name in ("staged_fp64", "pair_fp64", "fp32", "staged_fp64_fused", "pair_fp64_fused",
                     "fp32_fused"):
            e = plans["plain_fp64"][0].error_norms(res[name], ref)
            out[name]["max_rel_vs_plain"] = e["max_rel"]
        out["staged_fp64_fused"]["bit_equal_to_one_step_per_launch"] = bool(
            torch.equal(res["staged_fp64_fused"], res["staged_fp64"]))
        out["pair_fp64_fused"]["bit_equal_to_one_step_per_launch"] = bool(
            torch.equal(res["pair_fp64_fused"], res["pair_fp64"]))
        out["pair_fp64_fused"]["kernel"] = ("adv_ds_rows_fused (the 10 steps in one launch, "
                                            "two shared-memory copies of each line)")
        out["fp32_fused"]["bit_equal_to_one_step_per_launch"] = bool(
            torch.equal(res["fp32_fused"], res["fp32"]))
        out["speedup_staged_vs_plain"] = (out["staged_fp64"]["gcells_s"]
                                          / out["plain_fp64"]["gcells_s"])
        out["speedup_fused_fp64_vs_plain"] = (out["staged_fp64_fused"]["gcells_s"]
                                              / out["plain_fp64"]["gcells_s"])
        out["speedup_pair_vs_plain"] = (out["pair_fp64"]["gcells_s"]
                                        / out["plain_fp64"]["gcells_s"])
        out["speedup_pair_fused_vs_plain"] = (out["pair_fp64_fused"]["gcells_s"]
                                              / out["plain_fp64"]["gcells_s"])
        out["pair_fp64"]["kernel"] = ("adv_ds_rows (FP64 contiguous lines, FP32-pair "
                                      "arithmetic; the FP64 plans' default for n2 = 1)")
        v, c, el = cpu_adv_fields_sample(
            [dict(n0=n0, n1=n1, n2=n2, degree=5, ref=True, velocity=vel, dt=DT)],
            cores, n0, steps)
        reps = max(1, int(2.0 / max(el, 1e-3)))
        if reps > 1:
            v, c, el = cpu_adv_fields_sample(
                [dict(n0=n0, n1=n1, n2=n2, degree=5, ref=True, velocity=vel, dt=DT)],
                cores, n0, steps * reps)
        out["cpu_baseline"] = {"value": v, "unit": "GCells/s", "cores": cores, "kind": "port",
                               "sample": f"the whole workload, {steps * reps} steps, FP64, "
                                         f"{el:.2f} s"}
    except Exception as e:  # reported, not hidden
        out["error"] = repr(e)
    torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------------- GPU arm
def run_gpu(args):
    import numpy as np
    import torch
    import bkma_gb300

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    # weak scaling: each rank owns N0 velocity slabs of an (N0*world)-slab field
    n0_glob = N0 * world
    vel = velocities(n0_glob)[rank * N0:(rank + 1) * N0]
    kw = dict(dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0)
    plan = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f32", degree=5, weights="reference",
                                    velocity=vel, **kw)
    cells = N0 * N1 * N2
    f = torch.empty((N0, N1, N2), dtype=torch.float32, device=dev)
    plan.fill(f, mode=1, amp=NOISE, seed=SEED)
    if not args.no_autotune:
        plan.autotune(f)
        plan.fill(f, mode=1, amp=NOISE, seed=SEED)
    st = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.step(f)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local).start()
    barrier()
    torch.cuda.synchronize()
    t_start.record(st)
    for a, b in ev:
        a.record(st)
        plan.step(f)
        b.record(st)
    t_end.record(st)
    torch.cuda.synchronize()
    barrier()
    clocks = clk.stop()
    total_ms = t_start.elapsed_time(t_end)
    launch_ms = [a.elapsed_time(b) for a, b in ev]
    if dist is not None:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = cells * world * args.steps / (total_ms / 1e3) / 1e9
    hbm, _, peak_kind = peaks()
    avg_launch_s = statistics.mean(launch_ms) / 1e3
    achieved = cells * 8 / avg_launch_s / 1e9
    info = plan.info()
    kernel = {1: f"adv_tma_f32<6,{info['tile_cols']}>", 2: "adv_stream_f32<6>",
              3: "adv_rows_f32<6>"}.get(info["path"], "adv_staged<float,6>")
    traffic = None
    try:
        if (N0, N1, N2) == (2048, 1024, 512):
            with open(PROFILE_JSON[info["path"]]) as fp:
                traffic = json.load(fp).get("dram_bytes_per_launch")
    except Exception:
        pass
    del f
    torch.cuda.empty_cache()

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded sine + uniform noise, generated on the device)",
        "config": {"workload": WORKLOAD, "n0": N0, "n1": N1, "n2": N2, "degree": 5,
                   "dt": DT, "parallelism": f"replicas x{world} (n0 sharded, no exchange)",
                   "l2": "field 4 GiB > L2 129 MB, no flush",
                   "tile": {k: info[k] for k in ("tile_cols", "tile_slabs", "threads", "path",
                                                  "smem_bytes", "tiles", "exception_lines")}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "kernel": kernel,
                     "peak_kind": f"{peak_kind} copy bandwidth",
                     "algorithmic_bytes_per_launch": cells * 8},
        "gpu_launches": args.steps * (2 if info["path"] == 2 and info["exception_lines"] else 1),
        "clocks": clocks,
    }

    if rank == 0 and not args.quick:
        cores = os.cpu_count() or 1
        ext = extras(plan, bkma_gb300, dev, vel, kw, cells)
        # end to end first, on a quiet host (the CPU samples of the blocks
        # below load every host core)
        e2e_line = e2e(plan, dev, cells)
        result["config1"] = config1_block(bkma_gb300, dev, cores)
        result["conv1d"] = conv_block(bkma_gb300, dev, cores=cores)
        result["batched"] = batched_block(bkma_gb300, dev, cores=cores)
        result["learned"] = learned_block(bkma_gb300, dev, cores=cores)
        result["learned"]["under_resolved"] = under_resolved_block(bkma_gb300, dev)
        for k in ("fused_steps", "fp64_forms", "fused_hi_lo_50_steps"):
            result[k] = ext[k]
        result["e2e"] = e2e_line
        result["cpu_baseline"] = cpu_baseline_sample(cores)
        # last, so that a reader of the line's tail sees it
        result["error_vs_fp64"] = ext["error_vs_fp64"]
    if rank == 0:
        print(json.dumps(result))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def fused_block(bkma_gb300, dev, f, plan, vel, kw, cells):
    """Multi-step fusion, reported apart from the metric: k steps per launch
    on shared-memory strips cut HBM traffic to 8/k B per cell-step. Each k is
    checked bit for bit against `plan` (one step per launch) from field f."""
    import torch
    st = torch.cuda.current_stream()
    fz = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f32", velocity=vel, **kw)
    a1 = f.clone()
    plan.step(a1, nsteps=CFG_STEPS)
    fused = {}
    for k in (5, 10, 25):
        fz.set_fusion(k)
        a2 = f.clone()
        fz.step(a2, nsteps=CFG_STEPS)
        same = bool(torch.equal(a1, a2))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        fz.step(a2, nsteps=CFG_STEPS)
        b.record(st)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / CFG_STEPS
        fused[str(k)] = {"gcells_s": cells / (ms / 1e3) / 1e9, "hbm_bytes_per_cell_step": 8.0 / k,
                         "bit_identical_to_one_step_per_launch": same}
        del a2
    # hi + lo FP32 pair on chip: one FP32 rounding per launch
    fz.set_fused_state("f32x2")
    x2 = {}
    for k in (10, CFG_STEPS):
        fz.set_fusion(k)
        a2 = f.clone()
        fz.step(a2, nsteps=CFG_STEPS)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        fz.step(a2, nsteps=CFG_STEPS)
        b.record(st)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / CFG_STEPS
        x2[str(k)] = {"gcells_s": cells / (ms / 1e3) / 1e9, "hbm_bytes_per_cell_step": 8.0 / k}
        del a2
    del a1, fz
    return {"steps_per_launch": fused, "steps": CFG_STEPS,
            "kernel": "adv_fused_f32<6> (256 threads for n1 = 1024, 8-column strips, two shared buffers)",
            "hi_lo_state": {"steps_per_launch": x2,
                            "kernel": "adv_fused_f32x2<6,3> (352 threads for n1 = 1024, 4-column strips, hi + lo FP32 pair)"},
            "note": "not the metric: state stays in shared memory between steps"}


def fp64_block(bkma_gb300, dev, steps: int, warmup: int, tile_w: int = 0):
    """The FP64 plans' default kernel (FP32-pair arithmetic) alone on an
    N0 x N1 x N2 FP64 field (profiling captures): GCells/s over `steps` steps
    after `warmup`."""
    import torch
    vel = velocities(N0)
    kw = dict(dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0, velocity=vel)
    plan = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f64", **kw)
    if tile_w:
        plan.set_tile(tile_w, 1, 32 * tile_w, 4)
    d = torch.empty((N0, N1, N2), dtype=torch.float64, device=dev)
    plan.fill(d, mode=1, amp=NOISE, seed=SEED)
    plan.step(d, nsteps=warmup)
    st = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    plan.step(d, nsteps=steps)
    b.record(st)
    torch.cuda.synchronize()
    plan.status()
    ms = a.elapsed_time(b) / steps
    cells = N0 * N1 * N2
    return {"workload": f"FP64 advection {N0}x{N1}x{N2}, degree 5", "path": plan.info()["path"],
            "tile_cols": plan.info()["tile_cols"],
            "gcells_s": cells / (ms / 1e3) / 1e9, "ms_per_step": ms,
            "gbs": cells * 16 / (ms / 1e3) / 1e9}


def extras(plan, bkma_gb300, dev, vel, kw, cells):
    """Error of the 50-step FP32 run against the FP64 plain form (the
    reference's per-cell math, bit-identical to the oracle), and the speed of
    the FP64 forms on the same GPU."""
    import torch
    out = {}
    p64 = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f64", impl="plain", velocity=vel, **kw)
    s64 = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f64", velocity=vel, **kw)
    ref = torch.empty((N0, N1, N2), dtype=torch.float64, device=dev)
    p64.fill(ref, mode=1, amp=NOISE, seed=SEED)
    f = ref.float()
    ref = f.double()  # both start from the same FP32-representable field
    plan.step(f, nsteps=CFG_STEPS)
    st = torch.cuda.current_stream()

    def timed(pl, x, n):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        pl.step(x, nsteps=n)
        b.record(st)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    ms_plain = timed(p64, ref, CFG_STEPS)  # also produces the FP64 reference field
    norms = plan.error_norms(f, ref)
    one = {"max_rel_50": norms["max_rel"], "l2_rel_50": norms["l2_rel"]}
    # the same 50 steps in one launch with the hi + lo FP32 state on chip:
    # FP32 in HBM, rounded to FP32 once instead of 50 times
    g = torch.empty((N0, N1, N2), dtype=torch.float64, device=dev)
    p64.fill(g, mode=1, amp=NOISE, seed=SEED)
    x0 = g.float()
    del g
    fx = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f32", velocity=vel, **kw)
    fx.set_fused_state("f32x2")
    fx.set_fusion(CFG_STEPS)
    x1 = x0.clone()
    fx.step(x1, nsteps=CFG_STEPS)
    nx = plan.error_norms(x1, ref)
    ms_x2 = timed(fx, x0, CFG_STEPS)
    hilo = {"max_rel_50": nx["max_rel"], "l2_rel_50": nx["l2_rel"],
            "gcells_s": cells / (ms_x2 / 1e3) / 1e9}
    out["fused_hi_lo_50_steps"] = {
        "steps_per_launch": CFG_STEPS, "max_abs": nx["max_abs"], "max_rel": nx["max_rel"],
        "l2_rel": nx["l2_rel"], "gcells_s": cells / (ms_x2 / 1e3) / 1e9,
        "hbm_bytes_per_cell_step": 8.0 / CFG_STEPS,
        "kernel": "adv_fused_f32x2<6,3>",
        "note": "same field and 50 steps as the metric, FP32 in HBM; the cells stay on chip as "
                "an FP32 hi + lo pair between the steps of the launch; not the metric's "
                "one-step-per-launch roofline"}
    del x0, x1, fx
    # 10-step error as well (the FP32 storage floor grows with the step count)
    g = torch.empty((N0, N1, N2), dtype=torch.float64, device=dev)
    p64.fill(g, mode=1, amp=NOISE, seed=SEED)
    f10 = g.float()
    g.copy_(f10)
    g0 = g.clone()
    plan.step(f10, nsteps=10)
    p64.step(g, nsteps=10)
    n10 = plan.error_norms(f10, g)
    one.update({"max_rel_10": n10["max_rel"], "l2_rel_10": n10["l2_rel"]})
    out["error_vs_fp64"] = {
        "reference": "plain FP64 kernel (the reference's per-cell math, bit-exact with the "
                     "oracle), from the same FP32-representable field",
        "target_max_rel": 1e-6,
        "one_step_per_launch": one,
        "fused_hi_lo_50": hilo,
        "target_met_by": [k for k, v in (("one_step_per_launch", one), ("fused_hi_lo_50", hilo))
                          if v["max_rel_50"] <= 1e-6]}
    del f10
    # FP64 storage: the FP32-pair kernel (the FP64 plans' default) against the
    # FP64-arithmetic staged kernel and the plain form, 10 steps from the same field
    s64.set_tile(8, 1, 256, 0)
    d64 = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f64", velocity=vel, **kw)
    gd = g0
    d64.step(gd, nsteps=10)
    nd = p64.error_norms(gd, g)   # g: 10 plain FP64 steps
    gs = torch.empty_like(g)
    p64.fill(gs, mode=1, amp=NOISE, seed=SEED)
    gs.copy_(gs.float())
    s64.step(gs, nsteps=10)
    ns = p64.error_norms(gs, g)
    nds = p64.error_norms(gd, gs)
    del gs, g, gd, g0
    torch.cuda.empty_cache()
    ms_staged64 = timed(s64, ref, 10)
    ms_pair = []
    for _ in range(3):
        ms_pair.append(timed(d64, ref, 10))
    ms_pair64 = statistics.median(ms_pair)
    hbm, _, kind = peaks()
    f32ms = timed(plan, f, 10)
    pair_gcs = cells / (ms_pair64 / 1e3) / 1e9
    out["fp64_forms"] = {
        "plain_fp64_gcells_s": cells / (ms_plain / 1e3) / 1e9,
        "staged_fp64_gcells_s": cells / (ms_staged64 / 1e3) / 1e9,
        "pair_fp64_gcells_s": pair_gcs,
        "fp32_gcells_s": cells / (f32ms / 1e3) / 1e9,
        "speedup_vs_plain_fp64": ms_plain / f32ms,
        "speedup_vs_staged_fp64": ms_staged64 / f32ms,
        "pair_fp64": {
            "kernel": f"adv_ds_f64<6,{d64.info()['tile_cols']}> (FP64 in HBM, FP32-pair "
                      f"arithmetic, TMA tiles of {d64.info()['tile_cols']} columns)",
            "workload": "2048x1024x512 FP64, degree 5",
            "roofline": {"bound": "hbm", "achieved": pair_gcs * 16, "peak": hbm, "unit": "GB/s",
                         "frac": pair_gcs * 16 / hbm, "peak_kind": f"{kind} copy bandwidth",
                         "algorithmic_bytes_per_cell_step": 16},
            "speedup_vs_staged_fp64": ms_staged64 / ms_pair64,
            "speedup_vs_plain_fp64": ms_plain / ms_pair64,
            "max_rel_10_vs_plain": nd["max_rel"], "l2_rel_10_vs_plain": nd["l2_rel"],
            "max_rel_10_vs_staged_fp64": nds["max_rel"],
            "staged_fp64_max_rel_10_vs_plain": ns["max_rel"]},
    }
    out["fused_steps"] = fused_block(bkma_gb300, dev, f, plan, vel, kw, cells)
    del ref, f
    torch.cuda.empty_cache()
    return out


def conv_block(bkma_gb300, dev, batch: int = 256, with_fp64: bool = True, cores: int = 0):
    """In-place conv1d, BF16 with FP32 accumulation (tcgen05): B=256,
    Cin=Cout=128, L=8192, K=7, inputs and weights U[-1,1]/sqrt(Cin*K), bias 0.
    TFLOP/s = 2*B*Cout*Cin*K*(L-K+1) / kernel time; error against the plain
    FP64 kernel (bit-identical to the oracle) on the same BF16-rounded inputs,
    which is also the plain-FP64-form speed baseline."""
    import torch
    B, C, L, K = batch, 128, 8192, 7
    flops = 2.0 * B * C * C * K * (L - K + 1)
    out = {"workload": f"in-place conv1d BF16 B={B} Cin=Cout={C} L={L} K={K}",
           "metric": "conv1d TFLOP/s", "unit": "TFLOP/s"}
    try:
        g = torch.Generator(device=dev).manual_seed(SEED)
        s = 1.0 / (C * K) ** 0.5
        x0 = ((torch.rand((B, C, L), generator=g, device=dev) * 2 - 1) * s).to(torch.bfloat16)
        w = ((torch.rand((C, C, K), generator=g, device=dev) * 2 - 1) * s).to(torch.bfloat16)
        bias = torch.zeros(C, dtype=torch.bfloat16, device=dev)
        plan = bkma_gb300.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor")
        x = x0.clone()
        plan.run(x, w, bias)
        plan.status()
        st = torch.cuda.current_stream()
        reps = 20
        bufs = [x0.clone() for _ in range(2)]
        times = []
        for r in range(reps + 3):
            xb = bufs[r % 2]
            xb.copy_(x0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            plan.run(xb, w, bias)
            b.record(st)
            torch.cuda.synchronize()
            if r >= 3:
                times.append(a.elapsed_time(b))
        plan.status()
        ms = statistics.median(times)
        _, bf16_peak, kind = peaks()
        tflops = flops / (ms / 1e3) / 1e12
        out.update({"value": tflops, "ms": ms, "launches_per_call": 2,
                    "roofline": {"bound": "tensor", "achieved": tflops, "peak": bf16_peak,
                                 "unit": "TFLOP/s", "frac": tflops / bf16_peak,
                                 "peak_kind": f"{kind} cuBLAS bf16 burst",
                                 "algorithmic_flops": flops,
                                 "note": "time includes the prologue kernel (weight images + halo snapshot of each CTA's last tile)"}})
        if not with_fp64:
            raise StopIteration
        # FP64 plain form on the same BF16 inputs: error reference and speed baseline
        p64 = bkma_gb300.Conv1dPlan(B, C, C, L, K, dtype="f64", impl="plain")
        x64 = x0.double()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        p64.run(x64, w.double(), bias.double())
        b.record(st)
        torch.cuda.synchronize()
        ms64 = a.elapsed_time(b)
        got = x[:, :, :L - K + 1].double()
        ref = x64[:, :, :L - K + 1]
        d = (got - ref).abs()
        out["error_vs_fp64"] = {"max_rel": float(d.max() / ref.abs().max()),
                                "l2_rel": float((d.pow(2).sum() / ref.pow(2).sum()).sqrt())}
        out["plain_fp64"] = {"tflops": flops / (ms64 / 1e3) / 1e12, "ms": ms64,
                             "speedup": ms64 / ms}
        del x64, ref, got, d
        if cores:
            out["cpu_baseline"] = cpu_conv_sample(cores)
    except StopIteration:
        pass
    except Exception as e:  # reported, not hidden
        out["error"] = repr(e)
    torch.cuda.empty_cache()
    return out


def batched_block(bkma_gb300, dev, nfields: int = 64, steps: int = 10, autotune: bool = True,
                  cores: int = 0):
    """Batched uneven advection: 64 fields advanced by one graph launch per
    step (streamed kernels per tap count + the persistent staged kernel for
    what cannot stream), n0 ~ U{64..1024}, n1 in {256, 512, 1024, 2048}, n2 ~ U{1..256},
    FP32, degree 3 or 5 per field, line velocities ~ U[-2, 2], seeded
    sin(2 pi x) + U[-0.01, 0.01] init. GCells/s over all fields; roofline at
    8 B per cell-step against the measured HBM copy peak."""
    import numpy as np
    import torch
    out = {"workload": f"batched uneven advection, {nfields} fields, FP32, degree 3/5",
           "metric": "batched advection GCells/s", "unit": "GCells/s"}
    try:
        rng = np.random.default_rng(SEED)
        g = torch.Generator(device=dev).manual_seed(SEED)
        fields = []
        for _ in range(nfields):
            n0 = int(rng.integers(64, 1025))
            n1 = int(rng.choice([256, 512, 1024, 2048]))
            n2 = int(rng.integers(1, 257))
            deg = int(rng.choice([3, 5]))
            x = torch.arange(n1, device=dev, dtype=torch.float32) / n1
            d = torch.sin(2 * np.pi * x)[None, :, None] + NOISE * (
                2 * torch.rand((n0, n1, n2), generator=g, device=dev) - 1)
            fields.append(dict(data=d.contiguous(), degree=deg,
                               weights="reference" if deg == 5 else "lagrange", dt=DT,
                               minX=0.0, maxX=1.0, minVx=-2.0, maxVx=2.0,
                               velocity=rng.uniform(-2.0, 2.0, n0)))
        batch = bkma_gb300.AdvectionBatch(fields, dtype="f32")
        tiles = batch.autotune() if autotune else batch.tiles()
        st = torch.cuda.current_stream()
        batch.step(3)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        batch.step(steps)
        b.record(st)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / steps
        hbm, _, kind = peaks()
        gcs = batch.cells / (ms / 1e3) / 1e9
        out.update({"value": gcs, "ms_per_step": ms, "cells": batch.cells, "fields": nfields,
                    "launches_per_step": batch.launches_per_step(), "graph": True,
                    "streamed_fields": sum(1 for w in tiles["W"] if w == 0),
                    "tiles": {"count": tiles["tiles"], "threads": tiles["threads"],
                              "smem_bytes": tiles["smem_bytes"]},
                    "roofline": {"bound": "hbm", "achieved": gcs * 8, "peak": hbm,
                                 "unit": "GB/s", "frac": gcs * 8 / hbm,
                                 "peak_kind": f"{kind} copy bandwidth"}})
        spec = [dict(n0=f["data"].shape[0], n1=f["data"].shape[1], n2=f["data"].shape[2],
                     degree=f["degree"], ref=f["weights"] == "reference",
                     velocity=f["velocity"], dt=DT, minVx=-2.0, maxVx=2.0) for f in fields]
        del fields, batch
        torch.cuda.empty_cache()
        if cores:
            v, c, el = cpu_adv_fields_sample(spec, cores, 32, 3)
            out["cpu_baseline"] = {"value": v, "unit": "GCells/s", "cores": cores,
                                   "kind": "port",
                                   "sample": f"the first 32 velocity slabs of each of the "
                                             f"{nfields} fields, 3 steps ({c / 3:.3g} cells), "
                                             f"FP64, {el:.1f} s"}
    except Exception as e:  # reported, not hidden
        out["error"] = repr(e)
    torch.cuda.empty_cache()
    return out


def learned_block(bkma_gb300, dev, steps: int = 100, cores: int = 0):
    """Learned-stencil advection: the 4-point MLP stencil (1 -> 32 -> 32 -> 4,
    GELU, FP32) trained on the GPU on 10^6 (shift, degree-9 Lagrange) samples of
    random periodic lines (n1 = 1024), then applied to n0=1024 x n1=1024 x
    n2=256 FP32 for 100 steps, next to the plain degree-5 kernel and degree-3
    Lagrange (the same 4-point layout without the network). Accuracy is the RMS
    error against the exact shifted solution of a band-limited initial field."""
    import numpy as np
    import torch
    out = {"workload": "learned 4-point stencil vs degree 5 / degree 3, 1024x1024x256 FP32, "
                       "100 steps"}
    try:
        n0, n1, n2 = 1024, 1024, 256
        net = bkma_gb300.LearnedStencil(seed=SEED)
        a, f4, t = bkma_gb300.LearnedStencil.samples(1_000_000, SEED)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss = net.train(a, f4, t, steps=2000, batch=8192, lr=3e-3)
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0
        va, vf, vt = bkma_gb300.LearnedStencil.samples(1 << 18, SEED, first=1 << 30)
        w = net.infer(va)
        mse_l = float(((w * vf).sum(1) - vt).double().pow(2).mean())
        xs = 1.0 + va.double()
        l3 = torch.stack([((xs - m1) * (xs - m2) * (xs - m3)) / ((j - m1) * (j - m2) * (j - m3))
                          for j, (m1, m2, m3) in enumerate([(1, 2, 3), (0, 2, 3), (0, 1, 3),
                                                            (0, 1, 2)])], 1)
        mse_3 = float(((l3 * vf.double()).sum(1) - vt.double()).pow(2).mean())
        del a, f4, t, va, vf, vt
        vel = velocities(n0)
        rng = np.random.default_rng(SEED)
        modes = np.arange(1, 33)
        am = rng.uniform(-1, 1, modes.size) / modes
        bm = rng.uniform(-1, 1, modes.size) / modes

        def f(x):
            ph = 2 * np.pi * np.outer(x, modes)
            return (np.cos(ph) * am + np.sin(ph) * bm).sum(1)

        x = np.arange(n1) / n1
        init = torch.tensor(f(x), dtype=torch.float32, device=dev)
        kw = dict(dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0, velocity=vel)
        plans = {"learned_4pt": net.plan_for(n0, n1, n2, **kw),
                 "degree5_reference": bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f32", **kw),
                 "degree3_lagrange": bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f32", degree=3,
                                                              weights="lagrange", **kw)}
        sample = np.arange(0, n0, 64)
        st = torch.cuda.current_stream()
        for name, plan in plans.items():
            d = init[None, :, None].expand(n0, n1, n2).contiguous()
            plan.autotune(d)  # short lines: the default tile is not the fastest
            d.copy_(init[None, :, None].expand(n0, n1, n2))
            plan.step(d, nsteps=2)  # warm-up, then restart from the initial field
            d.copy_(init[None, :, None].expand(n0, n1, n2))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            plan.step(d, nsteps=steps)
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            got = d[sample, :, 0].double().cpu().numpy()
            err = 0.0
            for r, i0 in enumerate(sample):
                exact = f((x - vel[i0] * steps * DT) % 1.0)
                err += ((got[r] - exact) ** 2).mean()
            out[name] = {"gcells_s": n0 * n1 * n2 * steps / (ms / 1e3) / 1e9,
                         "rms_err_vs_exact": (err / len(sample)) ** 0.5}
            del d
        out["training"] = {"samples": 1_000_000, "steps": 2000, "batch": 8192, "seconds": train_s,
                           "last_batch_mse": loss, "held_out_mse_learned": mse_l,
                           "held_out_mse_degree3": mse_3, "mse_ratio": mse_l / mse_3}
        del plans
        torch.cuda.empty_cache()
        if cores:
            spec = [dict(n0=n0, n1=n1, n2=n2, degree=5, ref=True, velocity=vel, dt=DT)]
            v, c, el = cpu_adv_fields_sample(spec, cores, 512, 6)
            out["cpu_baseline"] = {"value": v, "unit": "GCells/s", "cores": cores,
                                   "kind": "port",
                                   "sample": f"degree 5 (the reference's method), 512 of {n0} "
                                             f"velocity slabs, 6 steps, FP64, {el:.1f} s"}
    except Exception as e:  # reported, not hidden
        out["error"] = repr(e)
    torch.cuda.empty_cache()
    return out


def under_resolved_block(bkma_gb300, dev, steps: int = 100):
    """Learned stencils where Lagrange is weak: a 32-mode periodic field on
    lines of n1 = 128 cells (half the grid's Nyquist band), n0 = 1024 velocity
    lines x n2 = 2048 columns FP32 (2^28 cells), dt = 0.001, 100 steps. The
    learned 6- and 4-point stencils are trained on the GPU on 2^20 samples of
    such lines with exact targets; all plans run the same FP32 kernels (TMA
    tiles), so the speed of a stencil depends only on its tap count. RMS error
    against the exact shifted solution on 16 sampled velocity lines."""
    import numpy as np
    import torch
    n0, n1, n2 = 1024, 128, 2048
    out = {"workload": f"learned 6/4-point vs degree 5/3 on under-resolved lines "
                       f"{n0}x{n1}x{n2} FP32, 32 modes, {steps} steps"}
    try:
        nets, train_s = {}, {}
        for npts in (6, 4):
            net = bkma_gb300.LearnedStencil(seed=SEED, npts=npts)
            a, f, t = bkma_gb300.LearnedStencil.samples(1 << 20, SEED, n1=n1, npts=npts, exact=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            net.train(a, f, t, steps=2000, batch=8192, lr=3e-3)
            torch.cuda.synchronize()
            train_s[npts] = time.perf_counter() - t0
            nets[npts] = net
            del a, f, t
        vel = velocities(n0)
        rng = np.random.default_rng(SEED + 1)
        modes = np.arange(1, 33)
        am = rng.uniform(-1, 1, modes.size) / modes
        bm = rng.uniform(-1, 1, modes.size) / modes

        def fx(x):
            ph = 2 * np.pi * np.outer(x, modes)
            return (np.cos(ph) * am + np.sin(ph) * bm).sum(1)

        x = np.arange(n1) / n1
        init = torch.tensor(fx(x), dtype=torch.float32, device=dev)
        kw = dict(dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0, velocity=vel)
        plans = {"learned_6pt": nets[6].plan_for(n0, n1, n2, **kw),
                 "degree5_reference": bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f32", **kw),
                 "degree5_lagrange": bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f32", degree=5,
                                                              weights="lagrange", **kw),
                 "learned_4pt": nets[4].plan_for(n0, n1, n2, **kw),
                 "degree3_lagrange": bkma_gb300.AdvectionPlan(n0, n1, n2, dtype="f32", degree=3,
                                                              weights="lagrange", **kw)}
        sample = np.arange(0, n0, 64)
        st = torch.cuda.current_stream()
        for name, plan in plans.items():
            d = init[None, :, None].expand(n0, n1, n2).contiguous()
            plan.autotune(d)  # short lines: the default tile is not the fastest
            d.copy_(init[None, :, None].expand(n0, n1, n2))
            plan.step(d, nsteps=2)  # warm-up, then restart from the initial field
            d.copy_(init[None, :, None].expand(n0, n1, n2))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            plan.step(d, nsteps=steps)
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            got = d[sample, :, 0].double().cpu().numpy()
            err = 0.0
            for r, i0 in enumerate(sample):
                exact = fx((x - vel[i0] * steps * DT) % 1.0)
                err += ((got[r] - exact) ** 2).mean()
            info = plan.info()
            out[name] = {"gcells_s": n0 * n1 * n2 * steps / (ms / 1e3) / 1e9,
                         "rms_err_vs_exact": (err / len(sample)) ** 0.5,
                         "tile": {k: info[k] for k in ("path", "tile_cols", "threads")}}
            del d
        out["training"] = {"samples": 1 << 20, "steps": 2000, "batch": 8192, "targets": "exact",
                           "seconds_6pt": train_s[6], "seconds_4pt": train_s[4]}
        out["learned6_error_ratio_vs_degree5"] = (out["learned_6pt"]["rms_err_vs_exact"]
                                                  / out["degree5_reference"]["rms_err_vs_exact"])
    except Exception as e:  # reported, not hidden
        out["error"] = repr(e)
    torch.cuda.empty_cache()
    return out


def e2e(plan, dev, cells):
    """The same metric through the C ABI with a HOST field: every e2e step
    copies the field host->device, runs the 50 time steps and copies it back
    (bkma_adv_run_host). Median of five steps (host-side stalls on a shared
    box show up as single slow steps); the pinned host<->device copy
    bandwidth of the same buffers is measured beside it."""
    import numpy as np
    import torch
    host = torch.empty((N0, N1, N2), dtype=torch.float32, pin_memory=True)
    d = torch.empty((N0, N1, N2), dtype=torch.float32, device=dev)
    nbytes = cells * 4
    link = {}
    for name, fn in (("h2d_gbs", lambda: d.copy_(host, non_blocking=True)),
                     ("d2h_gbs", lambda: host.copy_(d, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        link[name] = nbytes / (time.perf_counter() - t0) / 1e9
    plan.fill(d, mode=1, amp=NOISE, seed=SEED)
    host.copy_(d)
    del d
    torch.cuda.empty_cache()
    h = host.numpy()
    plan.run_host(h, nsteps=1)  # allocates the plan's device buffer
    torch.cuda.synchronize()
    per = []
    for _ in range(5):
        t0 = time.perf_counter()
        plan.run_host(h, nsteps=CFG_STEPS)
        per.append(cells * CFG_STEPS / (time.perf_counter() - t0) / 1e9)
    return {"value": statistics.median(per), "unit": UNIT, "steps_measured": per,
            "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
            "time_steps_per_transfer": CFG_STEPS, "pinned_copy": link,
            "note": "one e2e step = H2D of the field + 50 advection steps + D2H, "
                    "slab chunks pipelined: copies in on one stream, steps on two, copies out on one"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--quick", action="store_true", help="skip error/e2e/cpu/conv blocks")
    ap.add_argument("--n0", type=int, default=None, help="smaller field for profiling captures")
    ap.add_argument("--n1", type=int, default=None, help="other line length (profiling captures)")
    ap.add_argument("--n2", type=int, default=None, help="other column count (profiling captures)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--workload", default="advection",
                    choices=["advection", "conv", "batched", "learned", "fused", "fp64",
                             "config1"],
                    help="conv: only the conv1d block, as its own JSON line")
    ap.add_argument("--conv-batch", type=int, default=256, help="smaller batch for captures")
    ap.add_argument("--fields", type=int, default=64, help="batched workload: field count")
    ap.add_argument("--tile-w", type=int, default=0,
                    help="fp64 workload: tile width of the FP32-pair kernel (4 or 8)")
    args = ap.parse_args()
    global N0, N1, N2
    if args.n0:
        N0 = args.n0
    if args.n1:
        N1 = args.n1
    if args.n2:
        N2 = args.n2
    if args.n0 or args.n1 or args.n2:
        global WORKLOAD
        WORKLOAD = f"single advection FP32 {N0}x{N1}x{N2}, degree 5 (profiling shape)"
    if args.warmup < 3:
        args.warmup = 3
    if args.workload in ("batched", "learned", "fused", "fp64", "config1") and args.impl != "reference":
        import torch
        import bkma_gb300
        dev = torch.device("cuda", 0)
        if args.workload == "config1":
            r = config1_block(bkma_gb300, dev, os.cpu_count() or 1)
            print(json.dumps(r))
            return 0 if "error" not in r else 1
        if args.workload == "fp64":
            r = fp64_block(bkma_gb300, dev, args.steps, args.warmup, args.tile_w)
            print(json.dumps(r))
            return 0
        if args.workload == "fused":
            vel = velocities(N0)
            kw = dict(dt=DT, minX=MINX, maxX=MAXX, minVx=-1.0, maxVx=1.0)
            plan = bkma_gb300.AdvectionPlan(N0, N1, N2, dtype="f32", velocity=vel, **kw)
            f = torch.empty((N0, N1, N2), dtype=torch.float32, device=dev)
            plan.fill(f, mode=1, amp=NOISE, seed=SEED)
            r = {"workload": f"fused advection steps {N0}x{N1}x{N2} FP32, {CFG_STEPS} steps",
                 **fused_block(bkma_gb300, dev, f, plan, vel, kw, N0 * N1 * N2)}
            print(json.dumps(r))
            return 0
        if args.workload == "batched":
            r = batched_block(bkma_gb300, dev, nfields=args.fields,
                              autotune=not args.no_autotune)
        else:
            r = learned_block(bkma_gb300, dev)
            r["under_resolved"] = under_resolved_block(bkma_gb300, dev)
        print(json.dumps(r))
        return 0 if "error" not in r else 1
    if args.workload == "conv" and args.impl != "reference":
        import torch
        import bkma_gb300
        r = conv_block(bkma_gb300, torch.device("cuda", 0), batch=args.conv_batch,
                       with_fp64=not args.quick)
        print(json.dumps(r))
        return 0 if "error" not in r else 1
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
