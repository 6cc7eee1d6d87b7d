"""Advection parity on the GPU, through the C ABI, against the CPU oracle
(which tests/test_oracle_golden.py pins to the reference's own code).

Tolerances:
  - plain FP64 kernel: bit-exact (same operation order, no FMA contraction);
  - staged FP64 kernel: |err| <= 1e-11 * max|f| (per-line weights use the
    line's i1 = 0 fractional shift, which differs from the per-cell one by
    at most ~1e-12);
  - staged FP32 kernel: max |err| <= (3e-7 * steps + 2e-7) * max|f| against the
    FP64 oracle (FP32 storage rounding accumulates per step).
"""
import numpy as np
import pytest

from oracle import AdvParams

pytestmark = pytest.mark.gpu

CASES = [
    # n0, n1, n2, dt, minX, maxX, minVx, maxVx
    (8, 64, 3, 0.0010000000474974513, 0.0, 1.0, -1.0, 1.0),
    (5, 999, 2, 0.37, -0.5, 2.5, -3.0, 3.3),
    (16, 1024, 1, 1e-4, 0.0, 1.0, 0.0, 1.0),
    (4, 128, 17, 0.5, 0.0, 1.0, -4.0, 4.0),
    (3, 256, 64, 0.003, 0.0, 1.0, -1.0, 1.0),
    (2, 1000, 33, 0.0011, 0.0, 1.0, -1.0, 1.0),
]


def _init(p, seed=0):
    rng = np.random.default_rng(seed)
    x = p.minX + np.arange(p.n1) * ((p.maxX - p.minX) / p.n1)
    f = np.sin(2 * np.pi * (x - p.minX) / (p.maxX - p.minX))[None, :, None]
    f = f + 0.01 * rng.uniform(-1, 1, (p.n0, p.n1, p.n2))
    return np.ascontiguousarray(f)


def _plan(bkma, p, **kw):
    return bkma.AdvectionPlan(p.n0, p.n1, p.n2, dt=p.dt, minX=p.minX, maxX=p.maxX,
                              minVx=p.minVx, maxVx=p.maxVx, **kw)


def _to(cuda, a, dtype):
    import torch
    return torch.tensor(a, dtype=dtype, device=cuda)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("steps", [1, 3])
def test_plain_fp64_bitexact(bkma, cuda, oracle, case, steps):
    import torch
    p = AdvParams(*case)
    f0 = _init(p)
    plan = _plan(bkma, p, dtype="f64", impl="plain")
    d = _to(cuda, f0, torch.float64)
    plan.step(d, nsteps=steps)
    got = d.cpu().numpy()
    want = oracle.adv_step(p, f0.copy(), steps)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["small", "odd", "default"])
def test_plain_fp64_matches_reference_vectors(bkma, cuda, golden, name):
    import torch
    n0, n1, n2, dt, mnx, mxx, mnv, mxv = golden[f"adv_{name}_params"]
    p = AdvParams(int(n0), int(n1), int(n2), dt, mnx, mxx, mnv, mxv)
    plan = _plan(bkma, p, dtype="f64", impl="plain")
    d = _to(cuda, golden[f"adv_{name}_init"], torch.float64)
    done = 0
    for s in sorted(int(k.rsplit("step", 1)[1]) for k in golden if k.startswith(f"adv_{name}_step")):
        plan.step(d, nsteps=s - done)
        done = s
        assert np.array_equal(d.cpu().numpy(), golden[f"adv_{name}_step{s}"])


@pytest.mark.parametrize("case", CASES)
def test_staged_fp64_close(bkma, cuda, oracle, case):
    import torch
    p = AdvParams(*case)
    f0 = _init(p, 1)
    plan = _plan(bkma, p, dtype="f64")
    d = _to(cuda, f0, torch.float64)
    plan.step(d, nsteps=3)
    want = oracle.adv_step(p, f0.copy(), 3)
    err = np.abs(d.cpu().numpy() - want).max() / np.abs(want).max()
    assert err <= 1e-11, err


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("steps", [1, 10])
def test_staged_fp32_vs_fp64_oracle(bkma, cuda, oracle, case, steps):
    import torch
    p = AdvParams(*case)
    f0 = _init(p, 2).astype(np.float32).astype(np.float64)
    plan = _plan(bkma, p, dtype="f32")
    d = _to(cuda, f0, torch.float32)
    plan.step(d, nsteps=steps)
    want = oracle.adv_step(p, f0.copy(), steps)
    err = np.abs(d.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= 3e-7 * steps + 2e-7, err


@pytest.mark.parametrize("case", CASES)
def test_departure_offsets_bitexact(bkma, cuda, oracle, case):
    p = AdvParams(*case)
    plan = _plan(bkma, p, dtype="f32")
    offs, shifts = plan.line_table()
    n_exc = 0
    for i0 in range(p.n0):
        vx = oracle.line_velocity(p, i0)
        left0, d0 = oracle.departure(p, 0, vx)
        assert offs[i0] == (left0 - 2) % p.n1
        assert shifts[i0] == d0 - 2.0
        varying = any(((oracle.departure(p, i1, vx)[0] - 2 - i1) % p.n1) != offs[i0]
                      for i1 in range(p.n1))
        n_exc += int(varying)
    assert plan.info()["exception_lines"] == n_exc


def test_exception_lines_use_per_cell_stencils(bkma, cuda, oracle):
    """Lines whose departure offset changes along n1 (n1 = 1000 and
    whole-cell displacements): the per-cell tables must give the oracle's
    results."""
    import torch
    p = AdvParams(*EXC_CASE)
    plan = _plan(bkma, p, dtype="f64", velocity=EXC_VEL)
    assert plan.info()["exception_lines"] > 0
    f0 = _init(p, 3)
    d = _to(cuda, f0, torch.float64)
    plan.step(d, nsteps=2)
    want = oracle.adv_step(p, f0.copy(), 2, velocity=EXC_VEL)
    assert np.abs(d.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


# n1 = 1000 (dx inexact) and whole-cell displacements v*dt = k*dx: the
# departure cell's floor flips along n1, so these lines carry per-cell tables.
EXC_CASE = (6, 1000, 3, 0.001, 0.0, 1.0, -2.0, 3.0)
EXC_VEL = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])


@pytest.mark.parametrize("dtype", ["f32", "f64"])
@pytest.mark.parametrize("steps", [1, 2, 3])
def test_inplace_equals_out_of_place(bkma, cuda, dtype, steps):
    import torch
    p = AdvParams(*CASES[4])
    f0 = _init(p, 4)
    tdt = torch.float32 if dtype == "f32" else torch.float64
    plan = _plan(bkma, p, dtype=dtype)
    a = _to(cuda, f0, tdt)
    plan.step(a, nsteps=steps)
    src = _to(cuda, f0, tdt)
    out = torch.empty_like(src)
    plan.step(src, out=out, nsteps=steps)
    assert torch.equal(a, out)
    if steps == 1:
        assert torch.equal(src, _to(cuda, f0, tdt))


def test_sharded_equals_full(bkma, cuda):
    import torch
    p = AdvParams(*CASES[0])
    f0 = _init(p, 5)
    full = _plan(bkma, p, dtype="f32")
    a = _to(cuda, f0, torch.float32)
    full.step(a, nsteps=4)
    h = p.n0 // 2
    parts = []
    for off, cnt in ((0, h), (h, p.n0 - h)):
        sp = _plan(bkma, p, dtype="f32", i0_offset=off, i0_count=cnt)
        b = _to(cuda, f0[off:off + cnt], torch.float32)
        sp.step(b, nsteps=4)
        parts.append(b)
    assert torch.equal(a, torch.cat(parts, 0))


def test_velocity_array_and_degree3(bkma, cuda, oracle):
    import torch
    p = AdvParams(12, 256, 5, 0.001, 0.0, 1.0, -1.0, 1.0)
    vel = np.random.default_rng(6).uniform(-2, 2, p.n0)
    f0 = _init(p, 6)
    for degree, weights in ((5, "reference"), (3, "lagrange"), (5, "lagrange")):
        plan = _plan(bkma, p, dtype="f64", velocity=vel, degree=degree, weights=weights)
        d = _to(cuda, f0, torch.float64)
        plan.step(d, nsteps=2)
        want = oracle.adv_step(p, f0.copy(), 2, velocity=vel, degree=degree,
                               ref_weights=(weights == "reference"))
        assert np.abs(d.cpu().numpy() - want).max() <= 1e-11, (degree, weights)


def test_analytic_validation_on_device(bkma, cuda, oracle):
    """The reference's unit tests: fill sin(4 pi x), exact 0 at maxIter = 0,
    mean L1 < 1e-6 after each of 10 steps (validation_unittests.cpp:11-94)."""
    import torch
    p = AdvParams(16, 512, 4, 1e-4, 0.0, 1.0, 0.0, 1.0)
    plan = _plan(bkma, p, dtype="f64")
    d = torch.empty(p.n0, p.n1, p.n2, dtype=torch.float64, device=cuda)
    plan.fill(d, mode=0)
    hi, lo = plan.validate(d, 0)
    assert hi == 0.0 and lo == 0.0
    for it in range(1, 11):
        plan.step(d)
        hi, lo = plan.validate(d, it)
        assert hi < 1e-6
    # the device analytic check agrees with the oracle's
    ref = oracle.fill_adv(p)
    oracle.adv_step(p, ref, 10)
    assert abs(oracle.validate_adv(p, ref, 10) - hi) < 1e-9


def test_run_host_matches_device_path(bkma, cuda):
    import torch
    p = AdvParams(*CASES[3])
    f0 = _init(p, 7).astype(np.float32)
    plan = _plan(bkma, p, dtype="f32")
    d = _to(cuda, f0, torch.float32)
    plan.step(d, nsteps=3)
    h = f0.copy()
    plan.run_host(h, nsteps=3)
    assert np.array_equal(h, d.cpu().numpy())


@pytest.mark.parametrize("n2,velocity", [(512, None), (509, "exc")])
def test_run_host_pipeline_matches_device_path(bkma, cuda, n2, velocity):
    """A field of >= 256 MB goes through the chunked copy/compute pipeline
    (sub-plans over slab chunks on three streams): same bits as the device
    path, including exception lines and odd n2 (streamed kernel)."""
    import torch
    n0, n1 = 130, 1000
    p = AdvParams(n0, n1, n2, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = None
    if velocity == "exc":
        vel = np.resize(EXC_VEL, n0)
    plan = _plan(bkma, p, dtype="f32", velocity=vel)
    f0 = np.random.default_rng(8).uniform(-1, 1, (n0, n1, n2)).astype(np.float32)
    d = _to(cuda, f0, torch.float32)
    plan.step(d, nsteps=2)
    h = torch.from_numpy(f0.copy()).pin_memory()
    plan.run_host(h.numpy(), nsteps=2)
    assert np.array_equal(h.numpy(), d.cpu().numpy())
    del d
    torch.cuda.empty_cache()


def test_autotune_is_result_neutral(bkma, cuda):
    import torch
    p = AdvParams(6, 512, 48, 0.001, 0.0, 1.0, -1.0, 1.0)
    f0 = _init(p, 8)
    plan = _plan(bkma, p, dtype="f32")
    a = _to(cuda, f0, torch.float32)
    plan.step(a, nsteps=2)
    scratch = torch.empty_like(a)
    info = plan.autotune(scratch)
    assert info["autotuned"] == 1
    b = _to(cuda, f0, torch.float32)
    plan.step(b, nsteps=2)
    assert torch.equal(a, b)


def test_error_norms(bkma, cuda):
    import torch
    p = AdvParams(4, 64, 8, 0.001, 0.0, 1.0, -1.0, 1.0)
    plan = _plan(bkma, p, dtype="f32")
    rng = np.random.default_rng(9)
    ref = rng.standard_normal(plan.shape)
    x = (ref + 1e-3 * rng.standard_normal(plan.shape)).astype(np.float32)
    n = plan.error_norms(_to(cuda, x, torch.float32), _to(cuda, ref, torch.float64))
    d = x.astype(np.float64) - ref
    assert abs(n["max_abs"] - np.abs(d).max()) < 1e-12
    assert abs(n["max_ref"] - np.abs(ref).max()) < 1e-12
    assert abs(n["l2_rel"] - np.sqrt((d ** 2).sum() / (ref ** 2).sum())) < 1e-9


def test_zero_steps_is_identity(bkma, cuda):
    import torch
    p = AdvParams(*CASES[0])
    plan = _plan(bkma, p, dtype="f32")
    a = _to(cuda, _init(p), torch.float32)
    b = a.clone()
    plan.step(a, nsteps=0)
    assert torch.equal(a, b)


TMA_CASES = [
    (3, 256, 64, 0.003, 0.0, 1.0, -1.0, 1.0),
    (4, 1000, 48, 0.0011, 0.0, 1.0, -1.0, 1.0),   # last TMA box partly past n1
    (2, 300, 20, 0.002, 0.0, 1.0, -2.0, 2.0),     # ragged column block (16 + 4)
    (3, 64, 16, 0.01, 0.0, 1.0, -1.0, 1.0),
    (2, 2048, 32, 0.0007, 0.0, 1.0, -1.0, 1.0),
]


@pytest.mark.parametrize("case", TMA_CASES)
@pytest.mark.parametrize("degree,weights", [(5, "reference"), (3, "lagrange")])
def test_tma_and_cp_async_paths_bit_identical(bkma, cuda, oracle, case, degree, weights):
    """The TMA-staged kernel and the cp.async-staged kernel compute the same
    FP32 operations in the same order: identical bits, and both within the
    FP32 tolerance of the FP64 oracle."""
    import torch
    p = AdvParams(*case)
    f0 = _init(p, 10).astype(np.float32).astype(np.float64)
    outs = {}
    for path, W in ((0, 16), (1, 16), (1, 8)):
        if path == 1 and p.n2 < W:
            continue
        plan = _plan(bkma, p, dtype="f32", degree=degree, weights=weights)
        info = plan.set_tile(W, 1, 256, path)
        assert info["path"] == path
        d = _to(cuda, f0, torch.float32)
        plan.step(d, nsteps=3)
        plan.status()
        outs[(path, W)] = d
    ref = outs[(0, 16)]
    for k, v in outs.items():
        assert torch.equal(v, ref), k
    want = oracle.adv_step(p, f0.copy(), 3, degree=degree, ref_weights=(weights == "reference"))
    err = np.abs(ref.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= 3e-7 * 3 + 2e-7, err


def test_set_tile_validation(bkma, cuda):
    p = AdvParams(*TMA_CASES[0])
    plan = _plan(bkma, p, dtype="f32")
    with pytest.raises(bkma.BkmaError):
        plan.set_tile(16, 1, 100, 0)
    with pytest.raises(bkma.BkmaError):
        plan.set_tile(16, 2, 256, 0)
    f64 = _plan(bkma, p, dtype="f64")
    with pytest.raises(bkma.BkmaError):
        f64.set_tile(16, 1, 256, 1)


def _offset_field(cuda, f0, dtype, off):
    """A contiguous device copy of f0 that starts `off` elements into its
    allocation, so the field base sits anywhere inside a 16-byte chunk."""
    import torch
    buf = torch.zeros(f0.size + 4, dtype=dtype, device=cuda)
    v = buf[off:off + f0.size].view(f0.shape)
    v.copy_(torch.tensor(f0, dtype=dtype))
    return buf, v


STAGED_CASES = [
    (3, 256, 37, 0.003, 0.0, 1.0, -1.0, 1.0),   # odd n2: rows start anywhere in a chunk
    (2, 301, 50, 0.002, 0.0, 1.0, -2.0, 2.0),   # odd n1: halo rows off the chunk grid
    (4, 128, 64, 0.01, 0.0, 1.0, -1.0, 1.0),    # aligned rows: four-column compute
    (5, 77, 3, 0.004, 0.0, 1.0, -1.5, 1.5),     # whole-row tiles, several slabs each
    (40, 16, 1, 0.001, 0.0, 1.0, -1.0, 1.0),    # 16-cell slabs: several slabs at once
    (12, 16, 128, 0.002, 0.0, 1.0, -1.0, 1.0),  # short lines, wide rows
]


@pytest.mark.parametrize("case", STAGED_CASES)
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_staged_tiles_and_alignments_bit_identical(bkma, cuda, oracle, case, dtype):
    """The cp.async-staged kernel gives the same bits for every tile width,
    slab count, field alignment and in- or out-of-place step: staging only
    moves data and each cell's arithmetic is fixed."""
    import torch
    p = AdvParams(*case)
    tdt = torch.float32 if dtype == "f32" else torch.float64
    f0 = _init(p, 11)
    if dtype == "f32":
        f0 = f0.astype(np.float32).astype(np.float64)
    tiles = [(W, 1) for W in (4, 6, 8, 12, 16, 32) if W < p.n2]
    tiles += [(p.n2, 1), (p.n2, 2), (p.n2, 8)]
    esize = 4 if dtype == "f32" else 8
    tiles = [(W, R) for (W, R) in tiles if (p.n1 + 8) * (W + 2) * R * esize <= 200 * 1024]
    ref = None
    for (W, R) in tiles:
        for off in (0, 1, 3):
            plan = _plan(bkma, p, dtype=dtype)
            plan.set_tile(W, R, 256, 0)
            buf, d = _offset_field(cuda, f0, tdt, off)
            plan.step(d, nsteps=3)
            plan.status()
            got = d.cpu()
            if ref is None:
                ref = got
            assert torch.equal(got, ref), (W, R, off)
    # out of place, source and destination at different chunk offsets
    plan = _plan(bkma, p, dtype=dtype, inplace=False)
    plan.set_tile(8 if p.n2 > 8 else p.n2, 1, 256, 0)
    _, src = _offset_field(cuda, f0, tdt, 1)
    _, dst = _offset_field(cuda, np.zeros_like(f0), tdt, 2)
    plan.step(src, out=dst, nsteps=1)
    one = _plan(bkma, p, dtype=dtype)
    one.set_tile(8 if p.n2 > 8 else p.n2, 1, 256, 0)
    _, d1 = _offset_field(cuda, f0, tdt, 0)
    one.step(d1, nsteps=1)
    assert torch.equal(dst.cpu(), d1.cpu())
    want = oracle.adv_step(p, f0.copy(), 3)
    err = np.abs(ref.numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= (3e-7 * 3 + 2e-7 if dtype == "f32" else 1e-11), err


@pytest.mark.parametrize("off", [1, 3])
def test_plain_fp64_bitexact_unaligned(bkma, cuda, oracle, off):
    """The plain FP64 kernel stays bit-exact on a field that does not start
    on 16 bytes."""
    import torch
    p = AdvParams(*STAGED_CASES[1])
    f0 = _init(p, 12)
    plan = _plan(bkma, p, dtype="f64", impl="plain")
    _, d = _offset_field(cuda, f0, torch.float64, off)
    plan.step(d, nsteps=2)
    assert np.array_equal(d.cpu().numpy(), oracle.adv_step(p, f0.copy(), 2))


STREAM_CASES = [
    # (n0, n1, n2, dt, minX, maxX, minVx, maxVx), velocity or None
    ((4, 1024, 7, 0.001, 0.0, 1.0, -2.0, 2.0), None),       # odd n2, d of both signs
    ((3, 2048, 1, 0.0007, 0.0, 1.0, -2.0, 2.0), None),      # one column per line
    ((2, 100, 33, 0.01, 0.0, 1.0, -1.0, 1.0), None),        # n1 not a multiple of 16
    ((3, 64, 5, 0.004, 0.0, 1.0, -1.0, 1.0), None),         # shortest streamed n1
    ((4, 256, 64, 0.02, 0.0, 1.0, -1.0, 1.0), None),        # shifts of ~5 cells
    (EXC_CASE, EXC_VEL),                                    # exception lines (staged pass)
    # uneven row segments (n1 = 1030) and shifts near both ends of the window
    ((4, 1030, 5, 0.001, 0.0, 1.0, -20.0, 20.0), np.array([19.0, -17.5, 0.3, -0.3])),
]


@pytest.mark.parametrize("case,vel", STREAM_CASES)
@pytest.mark.parametrize("degree,weights", [(5, "reference"), (3, "lagrange"), (9, "lagrange")])
def test_streamed_path_bit_identical(bkma, cuda, oracle, case, vel, degree, weights):
    """The streamed kernel (each lane walks one column down the rows with a
    register window) gives the staged kernel's bits, in place from any base
    alignment and out of place, and stays within the FP32 tolerance of the
    FP64 oracle."""
    import torch
    p = AdvParams(*case)
    kw = dict(dtype="f32", degree=degree, weights=weights)
    if vel is not None:
        kw["velocity"] = vel
    f0 = _init(p, 21).astype(np.float32).astype(np.float64)
    ref_plan = _plan(bkma, p, **kw)
    ref_plan.set_tile(min(16, p.n2), 1, 256, 0)
    ref = _to(cuda, f0, torch.float32)
    ref_plan.step(ref, nsteps=3)
    plan = _plan(bkma, p, **kw)
    # row-segment modes: from the size, one segment, up to 2, up to 8
    for segs, off in ((0, 0), (1, 1), (2, 2), (8, 0), (8, 1)):
        info = plan.set_tile(16, segs, 256, 2)
        assert info["path"] == 2
        _, d = _offset_field(cuda, f0, torch.float32, off)
        plan.step(d, nsteps=3)
        plan.status()
        assert torch.equal(d, ref), (segs, off)
    oop = _plan(bkma, p, inplace=False, **kw)
    oop.set_tile(16, 8, 256, 2)
    _, src = _offset_field(cuda, f0, torch.float32, 3)
    dst = torch.zeros_like(src)
    oop.step(src, out=dst, nsteps=3)
    assert torch.equal(dst, ref)
    want = oracle.adv_step(p, f0.copy(), 3, degree=degree,
                           ref_weights=(weights == "reference"), velocity=vel)
    err = np.abs(ref.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= 3e-7 * 3 + 2e-7, err


def test_streamed_path_needs_small_shifts(bkma, cuda):
    """Lines whose per-step shift is beyond the streamed window keep the
    staged forms: the plan refuses the streamed path."""
    p = AdvParams(4, 256, 8, 0.37, 0.0, 1.0, -3.0, 3.3)
    plan = _plan(bkma, p, dtype="f32")
    with pytest.raises(bkma.BkmaError):
        plan.set_tile(16, 1, 256, 2)
    f64 = _plan(bkma, AdvParams(*STREAM_CASES[0][0]), dtype="f64")
    with pytest.raises(bkma.BkmaError):
        f64.set_tile(16, 1, 256, 2)


def test_short_lines_with_exception_lines(bkma, cuda, oracle):
    """n1 = 10 (dx inexact) with whole-cell displacements: exception lines
    inside multi-slab tiles of 10-cell slabs (several slabs per CTA pass)
    give the oracle's results, and every tile shape gives the same bits."""
    import torch
    p = AdvParams(5, 10, 3, 0.1, 0.0, 1.0, -1.0, 2.0)
    vel = np.array([1.0, 2.0, 0.5, -1.0, 0.3])
    f0 = _init(p, 13).astype(np.float32).astype(np.float64)
    outs = []
    for R in (1, 2, 5):
        plan = _plan(bkma, p, dtype="f32", velocity=vel)
        assert plan.info()["exception_lines"] == 2
        plan.set_tile(p.n2, R, 256, 0)
        d = _to(cuda, f0, torch.float32)
        plan.step(d, nsteps=3)
        outs.append(d.cpu())
    assert all(torch.equal(o, outs[0]) for o in outs)
    want = oracle.adv_step(p, f0.copy(), 3, velocity=vel)
    err = np.abs(outs[0].numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= 3e-7 * 3 + 2e-7, err


FUSED_CASES = [
    # (n0, n1, n2, dt, minX, maxX, minVx, maxVx), velocity or None
    ((4, 1024, 16, 0.001, 0.0, 1.0, -1.0, 1.0), None),
    ((3, 256, 37, 0.003, 0.0, 1.0, -2.0, 2.0), None),       # odd n2, ragged strip
    ((5, 77, 3, 0.004, 0.0, 1.0, -1.5, 1.5), None),         # narrow rows
    ((2, 2048, 20, 0.0007, 0.0, 1.0, -1.0, 1.0), None),     # 8-column strips
    (EXC_CASE, EXC_VEL),                                    # exception lines
]


@pytest.mark.parametrize("case,vel", FUSED_CASES)
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_fused_steps_bit_identical(bkma, cuda, oracle, case, vel, dtype):
    """k time steps per launch on strips held in shared memory give the bits
    of one step per launch, for any k and a step count that k does not
    divide; out of place, the input stays as it was."""
    import torch
    p = AdvParams(*case)
    tdt = torch.float32 if dtype == "f32" else torch.float64
    kw = dict(dtype=dtype)
    if vel is not None:
        kw["velocity"] = vel
    f0 = _init(p, 31)
    if dtype == "f32":
        f0 = f0.astype(np.float32).astype(np.float64)
    ref = _to(cuda, f0, tdt)
    one = _plan(bkma, p, **kw)
    if one.info()["path"] == 4:
        # FP64 fused steps compute in FP64: against the staged FP64 kernel, not
        # the default FP32-pair one
        one.set_tile(8, 1, 256, 0)
    one.step(ref, nsteps=7)
    for k in (2, 3, 7, 10):
        plan = _plan(bkma, p, **kw)
        plan.set_fusion(k)
        d = _to(cuda, f0, tdt)
        plan.step(d, nsteps=7)
        plan.status()
        assert torch.equal(d, ref), k
    oop = _plan(bkma, p, inplace=False, **kw)
    oop.set_fusion(3)
    src = _to(cuda, f0, tdt)
    out = torch.zeros_like(src)
    oop.step(src, out=out, nsteps=7)
    assert torch.equal(out, ref)
    assert torch.equal(src, _to(cuda, f0, tdt))
    want = oracle.adv_step(p, f0.copy(), 7, velocity=vel)
    err = np.abs(ref.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= (3e-7 * 7 + 2e-7 if dtype == "f32" else 1e-11), err


def test_fused_steps_limits(bkma, cuda):
    p = AdvParams(2, 64, 4, 0.001, 0.0, 1.0, -1.0, 1.0)
    with pytest.raises(bkma.BkmaError):
        _plan(bkma, p, dtype="f64", impl="plain").set_fusion(4)
    long_lines = AdvParams(2, 40000, 4, 0.001, 0.0, 1.0, -1.0, 1.0)
    with pytest.raises(bkma.BkmaError):
        _plan(bkma, long_lines, dtype="f32").set_fusion(4)
    with pytest.raises(bkma.BkmaError):
        _plan(bkma, p, dtype="f32").set_fusion(0)
    # FP32 lines longer than the fast strips hold: refused (slower than one
    # step per launch); FP64 keeps its one-column strips
    mid = AdvParams(2, 8192, 4, 0.001, 0.0, 1.0, -1.0, 1.0)
    with pytest.raises(bkma.BkmaError):
        _plan(bkma, mid, dtype="f32").set_fusion(4)
    _plan(bkma, mid, dtype="f64").set_fusion(4)


@pytest.mark.parametrize("case,vel", FUSED_CASES)
@pytest.mark.parametrize("degree", [3, 5, 9])
def test_fused_x2_one_step_per_launch_is_fp32(bkma, cuda, case, vel, degree):
    """With the hi + lo state and one step per launch, lo is zero when every
    step starts, and the arithmetic is the FP32 kernel's: same bits."""
    import torch
    p = AdvParams(*case)
    kw = dict(dtype="f32", degree=degree, weights="reference" if degree == 5 else "lagrange")
    if vel is not None:
        kw["velocity"] = vel
    f0 = _init(p, 41).astype(np.float32).astype(np.float64)
    ref = _to(cuda, f0, torch.float32)
    _plan(bkma, p, **kw).step(ref, nsteps=5)
    plan = _plan(bkma, p, **kw)
    plan.set_fused_state("f32x2")
    plan.set_fusion(4)
    d = _to(cuda, f0, torch.float32)
    for _ in range(5):
        plan.step(d, nsteps=1)
    plan.status()
    assert torch.equal(d, ref)


@pytest.mark.parametrize("case,vel", FUSED_CASES)
def test_fused_x2_rounds_once_per_launch(bkma, cuda, oracle, case, vel):
    """50 steps in one launch with the hi + lo state against the FP64 oracle:
    the error stays near one FP32 rounding (|f| <= 1.01: half an ulp is
    6e-8), below the error of 50 FP32 steps, each rounded to FP32; out of
    place the input stays as it was."""
    import torch
    p = AdvParams(*case)
    kw = dict(dtype="f32")
    if vel is not None:
        kw["velocity"] = vel
    f0 = _init(p, 43).astype(np.float32).astype(np.float64)
    want = oracle.adv_step(p, f0.copy(), 50, velocity=vel)
    scale = np.abs(want).max()
    std = _to(cuda, f0, torch.float32)
    _plan(bkma, p, **kw).step(std, nsteps=50)
    plan = _plan(bkma, p, inplace=False, **kw)
    plan.set_fused_state("f32x2")
    plan.set_fusion(50)
    src = _to(cuda, f0, torch.float32)
    out = torch.zeros_like(src)
    plan.step(src, out=out, nsteps=50)
    plan.status()
    assert torch.equal(src, _to(cuda, f0, torch.float32))
    err_x2 = np.abs(out.cpu().numpy().astype(np.float64) - want).max() / scale
    err_std = np.abs(std.cpu().numpy().astype(np.float64) - want).max() / scale
    assert err_x2 <= 2.5e-7, (err_x2, err_std)
    assert err_x2 < err_std, (err_x2, err_std)


def test_fused_x2_limits(bkma, cuda):
    p = AdvParams(2, 64, 4, 0.001, 0.0, 1.0, -1.0, 1.0)
    with pytest.raises(bkma.BkmaError):
        _plan(bkma, p, dtype="f64").set_fused_state("f32x2")
    long_lines = AdvParams(2, 4096, 4, 0.001, 0.0, 1.0, -1.0, 1.0)
    with pytest.raises(bkma.BkmaError):
        _plan(bkma, long_lines, dtype="f32").set_fused_state("f32x2")
    plan = _plan(bkma, p, dtype="f32")
    plan.set_fused_state("f32x2")
    plan.set_fused_state("f32")


ROWS_CASES = [
    # (n0, n1, n2, dt, minX, maxX, minVx, maxVx), velocity or None
    ((300, 16, 1, 0.001, 0.0, 1.0, -1.0, 1.0), None),     # the reference's 16-cell lines
    ((7, 1024, 1, 0.002, 0.0, 1.0, -2.0, 2.0), None),
    ((3, 4096, 1, 0.0007, 0.0, 1.0, -1.0, 1.0), None),
    ((5, 20, 1, 0.004, 0.0, 1.0, -3.0, 3.0), None),      # n1 not a power of two, shifts > 1 cell
    ((6, 1000, 1, 0.001, 0.0, 1.0, -2.0, 3.0), EXC_VEL),  # exception lines
    ((70000, 16, 1, 0.001, 0.0, 1.0, -1.0, 1.0), None),   # 274 CTAs of 256 lines
    ((600, 1024, 1, 0.001, 0.0, 1.0, -1.0, 1.0), None),   # 75 CTAs of 8 lines
]


@pytest.mark.parametrize("case,vel", ROWS_CASES)
@pytest.mark.parametrize("degree", [3, 5, 9])
def test_rows_path_bit_identical(bkma, cuda, case, vel, degree):
    """Contiguous-line kernel (n2 = 1, path 3) against the generic staged
    kernel on whole rows: same bits, for several lines per CTA (R that does
    not divide n0 leaves a partial last CTA)."""
    import torch
    p = AdvParams(*case)
    kw = dict(dtype="f32", degree=degree, weights="reference" if degree == 5 else "lagrange")
    if vel is not None:
        kw["velocity"] = vel
    f0 = _init(p, 51).astype(np.float32).astype(np.float64)
    ref = _to(cuda, f0, torch.float32)
    staged = _plan(bkma, p, **kw)
    staged.set_tile(1, 1, 256, 0)
    staged.step(ref, nsteps=3)
    plan = _plan(bkma, p, **kw)
    assert plan.info()["path"] == 3
    d = _to(cuda, f0, torch.float32)
    plan.step(d, nsteps=3)  # the default R
    plan.status()
    assert torch.equal(d, ref)
    for R in (1, 2, 64):
        plan.set_tile(1, max(1, min(R, p.n0, (200 * 1024) // (4 * p.n1))), 256, 3)
        d = _to(cuda, f0, torch.float32)
        plan.step(d, nsteps=3)
        plan.status()
        assert torch.equal(d, ref), R


def test_rows_path_misaligned_field_falls_back(bkma, cuda, oracle):
    """A field 4 bytes off the 16-byte grid runs the staged kernel instead
    (same bits), and both match the oracle within the FP32 bound."""
    import torch
    p = AdvParams(9, 64, 1, 0.003, 0.0, 1.0, -1.0, 1.0)
    f0 = _init(p, 52).astype(np.float32).astype(np.float64)
    plan = _plan(bkma, p, dtype="f32")
    assert plan.info()["path"] == 3
    aligned = _to(cuda, f0, torch.float32)
    plan.step(aligned, nsteps=2)
    buf = torch.zeros(f0.size + 4, dtype=torch.float32, device=cuda)
    off = buf[1:1 + f0.size].view(p.n0, p.n1, p.n2)
    off.copy_(_to(cuda, f0, torch.float32))
    plan.step(off, nsteps=2)
    plan.status()
    assert torch.equal(off, aligned)
    want = oracle.adv_step(p, f0.copy(), 2)
    err = np.abs(aligned.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= 3e-7 * 2 + 2e-7, err


def test_tensor_arguments_are_checked(bkma, cuda):
    """Host, mistyped, short and strided tensors are refused in Python with
    BKMA_ERR_INVALID_ARG before anything is launched; the field is untouched."""
    import torch
    plan = bkma.AdvectionPlan(8, 64, 4, dtype="f32")
    good = torch.ones((8, 64, 4), device=cuda)
    for bad, why in ((torch.ones((8, 64, 4)), "not a CUDA tensor"),
                     (torch.ones((8, 64, 4), device=cuda, dtype=torch.float64), "dtype"),
                     (torch.ones((7, 64, 4), device=cuda), "needed"),
                     (torch.ones((8, 4, 64), device=cuda).transpose(1, 2), "not contiguous")):
        with pytest.raises(bkma.BkmaError) as e:
            plan.step(bad)
        assert e.value.status == 1 and why in str(e.value)
    with pytest.raises(bkma.BkmaError):
        plan.step(good, out=torch.ones(10, device=cuda))
    conv = bkma.Conv1dPlan(2, 16, 16, 64, 3, dtype="bf16", impl="tensor")
    x = torch.ones((2, 16, 64), device=cuda, dtype=torch.bfloat16)
    with pytest.raises(bkma.BkmaError) as e:
        conv.run(x, torch.ones((16, 16, 2), device=cuda, dtype=torch.bfloat16))
    assert "weight" in str(e.value)
    torch.cuda.synchronize()
    assert torch.equal(good, torch.ones_like(good))
    assert torch.equal(x, torch.ones_like(x))
