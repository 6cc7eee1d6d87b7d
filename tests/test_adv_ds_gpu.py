"""FP64 advection in FP32-pair arithmetic (the FP64 plans' default kernels
where the shape allows it: degree 3 or 5 with column pairs of an even n2 >= 4
and n1 >= 128, whole slabs of shorter lines with an even n2, or contiguous
lines of n2 = 1 with n1 % 4 == 0), through the C ABI.

Tolerances:
  - against the staged FP64 kernel (FP64 direct form sum_k w_k f_k, the same
    per-line weights): |diff| <= 2e-13 * max|f| per step (each product of the
    pair arithmetic is exact, the sum carries ~48 bits);
  - against the oracle (the reference's per-cell FP64 math): 1e-11 * max|f|,
    the staged FP64 kernel's own bound (per-line weights);
  - tiles that hold a value the split cannot carry (|x| >= 2^126 or
    0 < |x| < 2^-74, subnormals, inf, NaN), exception lines and fields off
    the 16-byte grid run the staged kernel's FP64 arithmetic: bit-identical.
"""
import numpy as np
import pytest

from oracle import AdvParams

pytestmark = pytest.mark.gpu

DS_CASES = [
    # n0, n1, n2, dt, minX, maxX, minVx, maxVx
    (3, 256, 64, 0.003, 0.0, 1.0, -1.0, 1.0),
    (4, 1000, 10, 0.0011, 0.0, 1.0, -1.0, 1.0),   # 8 + 2 columns: ragged last tile
    (2, 2048, 16, 0.0007, 0.0, 1.0, -2.0, 2.0),
    (5, 300, 8, 0.02, 0.0, 1.0, -3.0, 3.0),       # shifts of several cells
    (3, 128, 24, 0.01, -0.5, 1.5, -1.0, 1.0),     # the shortest lines it is the default for
]
TOL = 2e-13


def _init(p, seed):
    rng = np.random.default_rng(seed)
    x = p.minX + np.arange(p.n1) * ((p.maxX - p.minX) / p.n1)
    f = np.sin(2 * np.pi * (x - p.minX) / (p.maxX - p.minX))[None, :, None]
    return np.ascontiguousarray(f + 0.01 * rng.uniform(-1, 1, (p.n0, p.n1, p.n2)))


def _plans(bkma, p, **kw):
    args = dict(dt=p.dt, minX=p.minX, maxX=p.maxX, minVx=p.minVx, maxVx=p.maxVx, dtype="f64")
    args.update(kw)
    ds = bkma.AdvectionPlan(p.n0, p.n1, p.n2, **args)
    st = bkma.AdvectionPlan(p.n0, p.n1, p.n2, **args)
    st.set_tile(8, 1, 256, 0)
    return ds, st


def test_ds_tile_widths_bit_identical(bkma, cuda):
    """4- and 8-column tiles run the same arithmetic per cell: same bits."""
    import torch
    p = AdvParams(*DS_CASES[1])
    f0 = _init(p, 9)
    ref = None
    for w in (4, 8):
        plan, _ = _plans(bkma, p)
        plan.set_tile(w, 1, 32 * w, 4)
        d = torch.tensor(f0, device=cuda)
        plan.step(d, nsteps=3)
        plan.status()
        if ref is None:
            ref = d
        else:
            assert torch.equal(d, ref)


@pytest.mark.parametrize("case", DS_CASES)
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_close_to_staged_and_oracle(bkma, cuda, oracle, case, degree):
    import torch
    p = AdvParams(*case)
    weights = "reference" if degree == 5 else "lagrange"
    ds, st = _plans(bkma, p, degree=degree, weights=weights)
    assert ds.info()["path"] == 4, ds.info()
    f0 = _init(p, 1)
    steps = 4
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=steps)
    st.step(b, nsteps=steps)
    ds.status()
    scale = b.abs().max().item()
    assert (a - b).abs().max().item() <= TOL * steps * scale
    want = oracle.adv_step(p, f0.copy(), steps, degree=degree, ref_weights=degree == 5)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_inplace_equals_out_of_place(bkma, cuda):
    import torch
    p = AdvParams(*DS_CASES[0])
    ds, _ = _plans(bkma, p)
    f0 = _init(p, 2)
    a = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=3)
    oop = bkma.AdvectionPlan(p.n0, p.n1, p.n2, dtype="f64", dt=p.dt, minVx=p.minVx,
                             maxVx=p.maxVx, inplace=False)
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(a, out)


@pytest.mark.parametrize("value", [1e200, -3e38 * 1e3, 1e-30, 5e-324, float("inf")])
def test_ds_unsplittable_value_runs_fp64(bkma, cuda, value):
    """A value the FP32 pair cannot carry sends every cell pair whose stencil
    reads it to the FP64 arithmetic: those cells equal the staged kernel bit
    for bit; every other cell stays within the pair arithmetic's bound."""
    import torch
    p = AdvParams(3, 256, 24, 0.003, 0.0, 1.0, -1.0, 1.0)
    ds, st = _plans(bkma, p)
    f0 = _init(p, 3)
    i0, r_bad, col = 1, 100, 11  # slab 1, column pair (10, 11)
    f0[i0, r_bad, col] = value
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a)
    st.step(b)
    ds.status()
    offs, _ = ds.line_table()
    npts = 6
    rows = [r for r in range(p.n1) if (r_bad - (r + int(offs[i0]))) % p.n1 < npts]
    assert len(rows) == npts
    pair = slice(col - col % 2, col - col % 2 + 2)
    hit = torch.zeros_like(a, dtype=torch.bool)
    hit[i0, rows, pair] = True
    assert torch.allclose(a[hit], b[hit], rtol=0, atol=0, equal_nan=True)
    diff = (a - b).abs()[~hit].max().item()
    assert diff <= TOL * b[~hit].abs().max().item()


def test_ds_zeros_and_sign_changes(bkma, cuda):
    """Exact zeros split exactly (a zero field stays zero); a field crossing
    zero with many tiny values stays within the bound."""
    import torch
    p = AdvParams(2, 512, 16, 0.001, 0.0, 1.0, -1.0, 1.0)
    ds, st = _plans(bkma, p)
    z = torch.zeros((p.n0, p.n1, p.n2), dtype=torch.float64, device=cuda)
    ds.step(z, nsteps=3)
    assert torch.count_nonzero(z).item() == 0
    x = np.arange(p.n1) / p.n1
    f0 = np.ascontiguousarray(np.broadcast_to((np.sin(2 * np.pi * x) ** 9)[None, :, None],
                                              (p.n0, p.n1, p.n2)))
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=5)
    st.step(b, nsteps=5)
    assert (a - b).abs().max().item() <= TOL * 5 * b.abs().max().item()


def test_ds_exception_lines_bit_identical_to_staged(bkma, cuda, oracle):
    """Lines whose departure offset varies along n1 use per-cell FP64
    stencils: the FP64 arithmetic, bit for bit."""
    import torch
    p = AdvParams(6, 1000, 8, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    ds, st = _plans(bkma, p, velocity=vel)
    assert ds.info()["exception_lines"] > 0 and ds.info()["path"] == 4
    f0 = _init(p, 4)
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=2)
    st.step(b, nsteps=2)
    exc = [i0 for i0 in range(p.n0)
           if len({(oracle.departure(p, i1, vel[i0])[0] - i1) % p.n1 for i1 in range(p.n1)}) > 1]
    assert exc and len(exc) == ds.info()["exception_lines"]
    for i0 in exc:
        assert torch.equal(a[i0], b[i0]), i0
    assert (a - b).abs().max().item() <= TOL * 2 * b.abs().max().item()


def test_ds_misaligned_field_runs_fp64(bkma, cuda):
    import torch
    p = AdvParams(*DS_CASES[0])
    ds, st = _plans(bkma, p)
    f0 = _init(p, 5)
    n = f0.size
    buf = torch.empty(n + 1, dtype=torch.float64, device=cuda)
    d = buf[1:].view(f0.shape)  # 8 bytes past a 16-byte boundary
    d.copy_(torch.tensor(f0, device=cuda))
    ds.step(d, nsteps=2)
    b = torch.tensor(f0, device=cuda)
    st.step(b, nsteps=2)
    assert torch.equal(d, b)


def test_ds_timeout_reported(bkma, cuda):
    import torch
    p = AdvParams(*DS_CASES[0])
    ds, st = _plans(bkma, p)
    f0 = torch.tensor(_init(p, 6), device=cuda)
    a = f0.clone()
    ds.set_wait_limit(0)
    ds.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        ds.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
    ds.set_wait_limit(1 << 22)
    ds.step(a)
    ds.status()
    b = f0.clone()
    ds2, _ = _plans(bkma, p)
    ds2.step(b)
    assert torch.equal(a, b)


def test_ds_autotune_keeps_the_pair_kernel(bkma, cuda):
    import torch
    p = AdvParams(*DS_CASES[2])
    ds, _ = _plans(bkma, p)
    f0 = torch.tensor(_init(p, 7), device=cuda)
    scratch = f0.clone()
    info = ds.autotune(scratch)
    assert info["path"] in (4, 6)  # the staged or streamed column pairs: the same bits
    a, b = f0.clone(), f0.clone()
    ds.step(a, nsteps=2)
    fresh, _ = _plans(bkma, p)
    fresh.step(b, nsteps=2)
    assert torch.equal(a, b)


# ---- contiguous lines (n2 = 1): the same arithmetic, 4 cells per thread (path 5)

ROWS_CASES = [
    # n0, n1, n2, dt, minX, maxX, minVx, maxVx
    (64, 1024, 1, 0.001, 0.0, 1.0, -1.0, 1.0),
    (16, 1000, 1, 0.0011, 0.0, 1.0, -1.0, 1.0),   # odd shifts of many lines, n1 % 8 != 0
    (300, 64, 1, 0.003, 0.0, 1.0, -2.0, 2.0),     # many short lines per CTA, ragged last CTA
    (9, 256, 1, 0.02, 0.0, 1.0, -3.0, 3.0),       # shifts of several cells
    (5, 16, 1, 0.01, -0.5, 1.5, -1.0, 1.0),       # the shortest lines the kernel takes
]


def _rows_plans(bkma, p, **kw):
    args = dict(dt=p.dt, minX=p.minX, maxX=p.maxX, minVx=p.minVx, maxVx=p.maxVx, dtype="f64")
    args.update(kw)
    ds = bkma.AdvectionPlan(p.n0, p.n1, p.n2, **args)
    st = bkma.AdvectionPlan(p.n0, p.n1, p.n2, **args)
    # the FP64-arithmetic staged kernel on whole rows (8 lines per CTA, fewer
    # for lines longer than 2048 cells)
    st.set_tile(1, max(1, min(8, 16384 // p.n1)), 256, 0)
    return ds, st


@pytest.mark.parametrize("case", ROWS_CASES)
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_rows_close_to_staged_and_oracle(bkma, cuda, oracle, case, degree):
    import torch
    p = AdvParams(*case)
    weights = "reference" if degree == 5 else "lagrange"
    ds, st = _rows_plans(bkma, p, degree=degree, weights=weights)
    assert ds.info()["path"] == 5, ds.info()
    f0 = _init(p, 11)
    steps = 4
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=steps)
    st.step(b, nsteps=steps)
    ds.status()
    scale = b.abs().max().item()
    assert (a - b).abs().max().item() <= TOL * steps * scale
    want = oracle.adv_step(p, f0.copy(), steps, degree=degree, ref_weights=degree == 5)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_rows_line_counts_bit_identical(bkma, cuda):
    """Any number of lines per CTA runs the same arithmetic per cell."""
    import torch
    p = AdvParams(*ROWS_CASES[2])
    f0 = _init(p, 12)
    ref = None
    for R in (1, 7, 64):
        plan, _ = _rows_plans(bkma, p)
        plan.set_tile(1, R, 256, 5)
        d = torch.tensor(f0, device=cuda)
        plan.step(d, nsteps=3)
        plan.status()
        if ref is None:
            ref = d
        else:
            assert torch.equal(d, ref)


def test_ds_rows_inplace_equals_out_of_place(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[0])
    ds, _ = _rows_plans(bkma, p)
    f0 = _init(p, 13)
    a = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=3)
    oop = bkma.AdvectionPlan(p.n0, p.n1, p.n2, dtype="f64", dt=p.dt, minVx=p.minVx,
                             maxVx=p.maxVx, inplace=False)
    assert oop.info()["path"] == 5
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(a, out)


@pytest.mark.parametrize("value", [1e200, 1e-30, float("inf")])
def test_ds_rows_unsplittable_value_runs_fp64(bkma, cuda, value):
    """Every cell whose stencil reads a value the pair cannot carry is computed
    in FP64 (the staged kernel's bits); the rest stay within the bound."""
    import torch
    p = AdvParams(4, 256, 1, 0.003, 0.0, 1.0, -1.0, 1.0)
    ds, st = _rows_plans(bkma, p)
    f0 = _init(p, 14)
    i0, r_bad = 2, 100
    f0[i0, r_bad, 0] = value
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a)
    st.step(b)
    ds.status()
    offs, _ = ds.line_table()
    rows = [r for r in range(p.n1) if (r_bad - (r + int(offs[i0]))) % p.n1 < 6]
    assert len(rows) == 6
    hit = torch.zeros_like(a, dtype=torch.bool)
    hit[i0, rows, 0] = True
    assert torch.allclose(a[hit], b[hit], rtol=0, atol=0, equal_nan=True)
    other = ~hit & torch.isfinite(b)
    diff = (a - b)[other].abs().max().item()
    assert diff <= TOL * b[other].abs().max().item()


def test_ds_rows_zero_field_stays_zero(bkma, cuda):
    import torch
    p = AdvParams(8, 512, 1, 0.001, 0.0, 1.0, -1.0, 1.0)
    ds, _ = _rows_plans(bkma, p)
    z = torch.zeros((p.n0, p.n1, p.n2), dtype=torch.float64, device=cuda)
    ds.step(z, nsteps=3)
    assert torch.count_nonzero(z).item() == 0


def test_ds_rows_exception_lines_bit_identical_to_staged(bkma, cuda, oracle):
    import torch
    p = AdvParams(6, 1000, 1, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    ds, st = _rows_plans(bkma, p, velocity=vel)
    assert ds.info()["exception_lines"] > 0 and ds.info()["path"] == 5
    f0 = _init(p, 15)
    a = torch.tensor(f0, device=cuda)
    b = torch.tensor(f0, device=cuda)
    ds.step(a, nsteps=2)
    st.step(b, nsteps=2)
    exc = [i0 for i0 in range(p.n0)
           if len({(oracle.departure(p, i1, vel[i0])[0] - i1) % p.n1 for i1 in range(p.n1)}) > 1]
    assert exc and len(exc) == ds.info()["exception_lines"]
    for i0 in exc:
        assert torch.equal(a[i0], b[i0]), i0
    assert (a - b).abs().max().item() <= TOL * 2 * b.abs().max().item()


def test_ds_rows_misaligned_field_runs_fp64(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[0])
    ds, st = _rows_plans(bkma, p)
    f0 = _init(p, 16)
    buf = torch.empty(f0.size + 1, dtype=torch.float64, device=cuda)
    d = buf[1:].view(f0.shape)  # 8 bytes past a 16-byte boundary
    d.copy_(torch.tensor(f0, device=cuda))
    ds.step(d, nsteps=2)
    b = torch.tensor(f0, device=cuda)
    st.step(b, nsteps=2)
    assert torch.equal(d, b)


def test_ds_rows_timeout_reported(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[0])
    ds, _ = _rows_plans(bkma, p)
    f0 = torch.tensor(_init(p, 17), device=cuda)
    a = f0.clone()
    ds.set_wait_limit(0)
    ds.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        ds.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
    ds.set_wait_limit(1 << 22)
    ds.step(a)
    ds.status()
    b = f0.clone()
    ds2, _ = _rows_plans(bkma, p)
    ds2.step(b)
    assert torch.equal(a, b)


def test_ds_rows_autotune_keeps_the_kernel(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[1])
    ds, _ = _rows_plans(bkma, p)
    f0 = torch.tensor(_init(p, 18), device=cuda)
    info = ds.autotune(f0.clone())
    assert info["path"] == 5
    a, b = f0.clone(), f0.clone()
    ds.step(a, nsteps=2)
    fresh, _ = _rows_plans(bkma, p)
    fresh.step(b, nsteps=2)
    assert torch.equal(a, b)


# ---- runs of 4-cell groups (W = 4): the 4-cell kernel's bits


@pytest.mark.parametrize("case", ROWS_CASES + [(3, 4096, 1, 0.0009, 0.0, 1.0, -1.0, 1.0)])
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_group_runs_bit_identical(bkma, cuda, case, degree):
    """Each thread walks consecutive 4-cell groups with sliding rings of
    raw and split taps: the 4-cell kernel's bits for any lines per CTA (runs
    of 1 to many groups, lines of 16 to 4096 cells, odd and even offsets), in
    place and out of place."""
    import torch
    p = AdvParams(*case)
    weights = "reference" if degree == 5 else "lagrange"
    f0 = _init(p, 49)
    ref, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
    ref.set_tile(1, 1, 256, 5)
    want = torch.tensor(f0, device=cuda)
    ref.step(want, nsteps=3)
    for R in sorted({1, 3, 8, min(64, p.n0)}):
        if R > p.n0 or R * p.n1 * 8 > 200 * 1024:
            continue
        g, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
        info = g.set_tile(4, R, 256, 5)
        assert info["path"] == 5 and info["tile_cols"] == 4
        d = torch.tensor(f0, device=cuda)
        g.step(d, nsteps=3)
        g.status()
        assert torch.equal(d, want), R
    oop, _ = _rows_plans(bkma, p, degree=degree, weights=weights, inplace=False)
    oop.set_tile(4, 1, 256, 5)
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(out, want)


def test_ds_group_runs_exception_lines_and_unsplittable(bkma, cuda):
    import torch
    p = AdvParams(6, 1000, 1, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    g, _ = _rows_plans(bkma, p, velocity=vel)
    g.set_tile(4, 2, 256, 5)
    assert g.info()["exception_lines"] > 0
    q, _ = _rows_plans(bkma, p, velocity=vel)
    q.set_tile(1, 2, 256, 5)
    f0 = _init(p, 50)
    f0[1, 501, 0] = 1e200
    f0[3, 7, 0] = 5e-324
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    g.step(a, nsteps=2)
    q.step(b, nsteps=2)
    g.status()
    assert torch.allclose(a, b, rtol=0, atol=0, equal_nan=True)


def test_ds_group_runs_timeout_reported(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[0])
    g, _ = _rows_plans(bkma, p)
    g.set_tile(4, 8, 256, 5)
    f0 = torch.tensor(_init(p, 51), device=cuda)
    a = f0.clone()
    g.set_wait_limit(0)
    g.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        g.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)


# ---- short lines shared by a warp's lanes (W = 5): the 4-cell kernel's bits


@pytest.mark.parametrize("n1", [16, 32, 64, 128])
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_lineq_bit_identical(bkma, cuda, n1, degree):
    """The lanes of a line split its taps once each and exchange them by
    shuffles: the 4-cell kernel's bits for any lines per CTA, with a ragged
    last CTA (whole warps run the shuffles, lanes past the lines store
    nothing), in place and out of place."""
    import torch
    p = AdvParams(37, n1, 1, 0.003, 0.0, 1.0, -2.0, 2.0)
    weights = "reference" if degree == 5 else "lagrange"
    f0 = _init(p, 52)
    ref, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
    ref.set_tile(1, 1, 256, 5)
    want = torch.tensor(f0, device=cuda)
    ref.step(want, nsteps=3)
    for R in (1, 3, 8, 37):
        g, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
        info = g.set_tile(5, R, 256, 5)
        assert info["path"] == 5 and info["tile_cols"] == 5
        d = torch.tensor(f0, device=cuda)
        g.step(d, nsteps=3)
        g.status()
        assert torch.equal(d, want), R
    oop, _ = _rows_plans(bkma, p, degree=degree, weights=weights, inplace=False)
    oop.set_tile(5, 8, 256, 5)
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(out, want)


def test_ds_lineq_exception_lines_and_unsplittable(bkma, cuda, oracle):
    import torch
    n1 = 64
    # dx = 1.1 / n1 is inexact: whole-cell shifts give exception lines
    p = AdvParams(9, n1, 1, 1.1 / n1, 0.0, 1.1, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77, 2.0, -1.0, 0.1])
    g, _ = _rows_plans(bkma, p, velocity=vel)
    g.set_tile(5, 4, 256, 5)
    q, _ = _rows_plans(bkma, p, velocity=vel)
    q.set_tile(1, 4, 256, 5)
    f0 = _init(p, 53)
    f0[4, 10, 0] = 1e200
    f0[7, 63, 0] = float("inf")
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    g.step(a, nsteps=2)
    q.step(b, nsteps=2)
    g.status()
    assert torch.allclose(a, b, rtol=0, atol=0, equal_nan=True)
    f1 = _init(p, 54)
    c = torch.tensor(f1, device=cuda)
    g.step(c, nsteps=2)
    want = oracle.adv_step(p, f1.copy(), 2, velocity=vel)
    assert np.abs(c.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_lineq_timeout_reported(bkma, cuda):
    """A staging wait that gives up: every lane still leaves through the same
    path (no shuffle left waiting), the status reports the timeout and the
    field is untouched."""
    import torch
    p = AdvParams(40, 64, 1, 0.003, 0.0, 1.0, -2.0, 2.0)
    g, _ = _rows_plans(bkma, p)
    g.set_tile(5, 8, 256, 5)
    f0 = torch.tensor(_init(p, 57), device=cuda)
    a = f0.clone()
    g.set_wait_limit(0)
    g.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        g.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
    g.set_wait_limit(1 << 22)
    g.step(a)
    g.status()
    q, _ = _rows_plans(bkma, p)
    q.set_tile(1, 8, 256, 5)
    b = f0.clone()
    q.step(b)
    assert torch.equal(a, b)


# ---- lines of 8192 cells and more: half lines in 2-CTA clusters (W = 3)


@pytest.mark.parametrize("n1", [8192, 16384])
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_halves_bit_identical(bkma, cuda, oracle, n1, degree):
    """Each CTA of a cluster stages only its half line's window and writes
    its half after the cluster barrier: the 4-cell and run kernels' bits, in
    place and out of place."""
    import torch
    p = AdvParams(7, n1, 1, 0.0013, 0.0, 1.0, -2.0, 2.0)
    weights = "reference" if degree == 5 else "lagrange"
    f0 = _init(p, 45)
    outs = []
    for W, R in ((3, 1), (1, 1), (2, 1), (6, 1)):
        ds, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
        info = ds.set_tile(W, R, 256, 5)
        if W in (3, 6):
            assert info["tile_cols"] == W and info["tiles"] == 2 * p.n0, info
        d = torch.tensor(f0, device=cuda)
        ds.step(d, nsteps=3)
        ds.status()
        outs.append(d)
    for o in outs[1:]:
        assert torch.equal(outs[0], o)
    oop, _ = _rows_plans(bkma, p, degree=degree, weights=weights, inplace=False)
    oop.set_tile(6, 1, 256, 5)
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(out, outs[0])
    want = oracle.adv_step(p, f0.copy(), 3, degree=degree, ref_weights=degree == 5)
    assert np.abs(outs[0].cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_halves_default_for_long_lines(bkma, cuda):
    """Lines of 16384 cells (128 KB, one CTA per SM whole) default to half
    lines once there are enough lines to fill the GPU."""
    p = AdvParams(160, 16384, 1, 0.001, 0.0, 1.0, -1.0, 1.0)
    ds, _ = _rows_plans(bkma, p)
    info = ds.info()
    assert info["path"] == 5 and info["tile_cols"] == 6, info


@pytest.mark.parametrize("W", [3, 6])
def test_ds_halves_exception_lines_and_unsplittable(bkma, cuda, oracle, W):
    """Exception lines (offsets one cell either side of the line's) stay
    within the staged window; windows the pair cannot carry take FP64 (W = 3:
    runs along the two quarters, W = 6: runs of 4-cell groups)."""
    import torch
    n1 = 16384
    # dx = 1.1 / n1 is inexact: the lines shifted by whole cells (v = -2, 3)
    # have offsets one cell apart along n1
    p = AdvParams(6, n1, 1, 1.1 / n1, 0.0, 1.1, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    hv, _ = _rows_plans(bkma, p, velocity=vel)
    hv.set_tile(W, 1, 256, 5)
    assert hv.info()["exception_lines"] > 0
    q, _ = _rows_plans(bkma, p, velocity=vel)
    q.set_tile(1, 1, 256, 5)
    f0 = _init(p, 46)
    f0[2, 8190, 0] = 1e200  # near the seam between the two halves
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    hv.step(a, nsteps=2)
    q.step(b, nsteps=2)
    hv.status()
    assert torch.allclose(a, b, rtol=0, atol=0, equal_nan=True)
    f1 = _init(p, 47)
    c = torch.tensor(f1, device=cuda)
    hv.step(c, nsteps=2)
    want = oracle.adv_step(p, f1.copy(), 2, velocity=vel)
    assert np.abs(c.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_halves_autotune_keeps_the_bits(bkma, cuda):
    """The tuner times every line form for 16384-cell lines (both half-line
    cluster forms among them): whichever wins, the bits are the default's."""
    import torch
    p = AdvParams(4, 16384, 1, 0.0013, 0.0, 1.0, -2.0, 2.0)
    ds, _ = _rows_plans(bkma, p)
    f0 = torch.tensor(_init(p, 55), device=cuda)
    info = ds.autotune(f0.clone())
    assert info["path"] == 5, info
    a, b = f0.clone(), f0.clone()
    ds.step(a, nsteps=2)
    ds.status()
    fresh, _ = _rows_plans(bkma, p)
    fresh.step(b, nsteps=2)
    assert torch.equal(a, b), info


@pytest.mark.parametrize("W", [3, 6])
def test_ds_halves_timeout_reported(bkma, cuda, W):
    """A staging wait that gives up still reaches the cluster barrier: the
    call returns, the status reports the timeout and the field is untouched."""
    import torch
    p = AdvParams(4, 16384, 1, 0.001, 0.0, 1.0, -1.0, 1.0)
    hv, _ = _rows_plans(bkma, p)
    hv.set_tile(W, 1, 256, 5)
    f0 = torch.tensor(_init(p, 48), device=cuda)
    a = f0.clone()
    hv.set_wait_limit(0)
    hv.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        hv.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
    hv.set_wait_limit(1 << 22)
    hv.step(a)
    hv.status()
    q, _ = _rows_plans(bkma, p)
    q.set_tile(1, 1, 256, 5)
    b = f0.clone()
    q.step(b)
    assert torch.equal(a, b)


# ---- contiguous lines, k steps per launch in the same arithmetic


@pytest.mark.parametrize("case", ROWS_CASES)
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_rows_fused_bit_identical(bkma, cuda, case, degree):
    """k fused steps per launch (two shared-memory copies of each line) give
    the bits of one step per launch of the FP32-pair kernel, for any k and a
    step count k does not divide; out of place, the input stays as it was."""
    import torch
    p = AdvParams(*case)
    weights = "reference" if degree == 5 else "lagrange"
    one, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
    assert one.info()["path"] == 5
    f0 = _init(p, 40)
    ref = torch.tensor(f0, device=cuda)
    one.step(ref, nsteps=7)
    for k in (2, 3, 7, 10):
        fz, _ = _rows_plans(bkma, p, degree=degree, weights=weights)
        fz.set_fusion(k)
        d = torch.tensor(f0, device=cuda)
        fz.step(d, nsteps=7)
        fz.status()
        assert torch.equal(d, ref), k
    oop, _ = _rows_plans(bkma, p, degree=degree, weights=weights, inplace=False)
    oop.set_fusion(3)
    src = torch.tensor(f0, device=cuda)
    out = torch.zeros_like(src)
    oop.step(src, out=out, nsteps=7)
    assert torch.equal(out, ref)
    assert torch.equal(src, torch.tensor(f0, device=cuda))


def test_ds_rows_fused_exception_lines_and_unsplittable(bkma, cuda, oracle):
    """Exception lines and windows the pair cannot carry take the FP64
    arithmetic in every fused step, as in one step per launch."""
    import torch
    p = AdvParams(6, 1000, 1, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    one, _ = _rows_plans(bkma, p, velocity=vel)
    assert one.info()["exception_lines"] > 0
    f0 = _init(p, 41)
    f0[1, 500, 0] = 1e200
    ref = torch.tensor(f0, device=cuda)
    one.step(ref, nsteps=5)
    fz, _ = _rows_plans(bkma, p, velocity=vel)
    fz.set_fusion(5)
    d = torch.tensor(f0, device=cuda)
    fz.step(d, nsteps=5)
    fz.status()
    assert torch.allclose(d, ref, rtol=0, atol=0, equal_nan=True)
    f1 = _init(p, 42)
    want = oracle.adv_step(p, f1.copy(), 5, velocity=vel)
    e = torch.tensor(f1, device=cuda)
    fz.step(e, nsteps=5)
    assert np.abs(e.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_rows_fused_misaligned_field_runs_fp64(bkma, cuda):
    """A field off the 16-byte grid runs the FP64 staged arithmetic, fused or
    not: the same bits either way."""
    import torch
    p = AdvParams(*ROWS_CASES[0])
    one, _ = _rows_plans(bkma, p)
    fz, _ = _rows_plans(bkma, p)
    fz.set_fusion(4)
    f0 = _init(p, 43)
    views = []
    for _ in range(2):
        buf = torch.empty(f0.size + 1, dtype=torch.float64, device=cuda)
        d = buf[1:].view(f0.shape)  # 8 bytes past a 16-byte boundary
        d.copy_(torch.tensor(f0, device=cuda))
        views.append(d)
    one.step(views[0], nsteps=4)
    fz.step(views[1], nsteps=4)
    assert torch.equal(views[0], views[1])


def test_ds_rows_fused_timeout_reported(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[0])
    fz, _ = _rows_plans(bkma, p)
    fz.set_fusion(4)
    f0 = torch.tensor(_init(p, 44), device=cuda)
    a = f0.clone()
    fz.set_wait_limit(0)
    fz.step(a, nsteps=4)
    with pytest.raises(bkma.BkmaError) as e:
        fz.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
    fz.set_wait_limit(1 << 22)
    fz.step(a, nsteps=4)
    fz.status()
    one, _ = _rows_plans(bkma, p)
    b = f0.clone()
    one.step(b, nsteps=4)
    assert torch.equal(a, b)


# ---- whole slabs of short lines (n1 < 128, even n2): column pairs down
# whole lines (path 5 with n2 > 1), the column-pair kernel's bits

SLAB_CASES = [
    # n0, n1, n2, dt, minX, maxX, minVx, maxVx
    (64, 16, 128, 0.001, 0.0, 1.0, -1.0, 1.0),   # the reference's 2^20 x 16 x 128 sweep shape
    (17, 64, 24, 0.004, 0.0, 1.0, -2.0, 2.0),    # a last CTA with fewer slabs
    (40, 48, 6, 0.01, 0.0, 1.0, -3.0, 3.0),      # three pairs per slab: a warp spans slabs
    (9, 100, 4, 0.02, -0.5, 1.5, -1.0, 1.0),     # shifts of several cells
]


def _slab_plans(bkma, p, **kw):
    ds, st = _plans(bkma, p, **kw)
    col = bkma.AdvectionPlan(p.n0, p.n1, p.n2, dt=p.dt, minX=p.minX, maxX=p.maxX,
                             minVx=p.minVx, maxVx=p.maxVx, dtype="f64", **kw)
    col.set_tile(4, 1, 128, 4)
    return ds, st, col


@pytest.mark.parametrize("case", SLAB_CASES)
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_slabs_equal_column_pair_kernel(bkma, cuda, oracle, case, degree):
    """Lines shorter than 128 rows with an even n2 default to whole slabs:
    the column-pair kernel's bits, within the bound of the staged FP64
    kernel and the oracle."""
    import torch
    p = AdvParams(*case)
    weights = "reference" if degree == 5 else "lagrange"
    ds, st, col = _slab_plans(bkma, p, degree=degree, weights=weights)
    assert ds.info()["path"] == 5, ds.info()
    f0 = _init(p, 32)
    steps = 3
    a, b, c = (torch.tensor(f0, device=cuda) for _ in range(3))
    ds.step(a, nsteps=steps)
    col.step(b, nsteps=steps)
    st.step(c, nsteps=steps)
    ds.status()
    assert torch.equal(a, b)
    assert (a - c).abs().max().item() <= TOL * steps * c.abs().max().item()
    want = oracle.adv_step(p, f0.copy(), steps, degree=degree, ref_weights=degree == 5)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_ds_slabs_per_cta_bit_identical(bkma, cuda):
    """Any number of slabs per CTA and of runs per column pair (W), in place
    or out of place: the same bits."""
    import torch
    p = AdvParams(*SLAB_CASES[1])
    f0 = _init(p, 33)
    ref = None
    for R, runs in ((1, 1), (2, 1), (3, 2), (8, 4), (1, 8), (5, 3), (2, 64)):
        ds, _, _ = _slab_plans(bkma, p)
        ds.set_tile(runs, R, 256, 5)
        d = torch.tensor(f0, device=cuda)
        ds.step(d, nsteps=2)
        ds.status()
        ref = d if ref is None else ref
        assert torch.equal(d, ref), (R, runs)
    oop, _, _ = _slab_plans(bkma, p, inplace=False)
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=2)
    assert torch.equal(out, ref)


@pytest.mark.parametrize("value", [1e200, 1e-30, float("inf")])
def test_ds_slabs_unsplittable_value_runs_fp64(bkma, cuda, value):
    import torch
    p = AdvParams(*SLAB_CASES[1])
    ds, _, col = _slab_plans(bkma, p)
    f0 = _init(p, 34)
    f0[3, 40, 11] = value
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    ds.step(a)
    col.step(b)
    ds.status()
    assert torch.allclose(a, b, rtol=0, atol=0, equal_nan=True)


def test_ds_slabs_exception_lines_bit_identical(bkma, cuda):
    """n1 = 100 with whole-cell displacements: exception lines run the staged
    kernel's per-cell FP64 arithmetic."""
    import torch
    p = AdvParams(6, 100, 8, 0.01, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    ds, st, col = _slab_plans(bkma, p, velocity=vel)
    assert ds.info()["exception_lines"] > 0 and ds.info()["path"] == 5
    f0 = _init(p, 35)
    a, b, c = (torch.tensor(f0, device=cuda) for _ in range(3))
    ds.step(a, nsteps=2)
    col.step(b, nsteps=2)
    st.step(c, nsteps=2)
    ds.status()
    assert torch.equal(a, b)
    assert (a - c).abs().max().item() <= TOL * 2 * c.abs().max().item()


def test_ds_slabs_misaligned_field_runs_fp64(bkma, cuda):
    import torch
    p = AdvParams(*SLAB_CASES[0])
    ds, st, _ = _slab_plans(bkma, p)
    f0 = _init(p, 36)
    buf = torch.empty(f0.size + 1, dtype=torch.float64, device=cuda)
    d = buf[1:].view(f0.shape)  # 8 bytes past a 16-byte boundary
    d.copy_(torch.tensor(f0, device=cuda))
    ds.step(d, nsteps=2)
    b = torch.tensor(f0, device=cuda)
    st.step(b, nsteps=2)
    assert torch.equal(d, b)


def test_ds_slabs_timeout_reported(bkma, cuda):
    import torch
    p = AdvParams(*SLAB_CASES[0])
    ds, _, col = _slab_plans(bkma, p)
    f0 = torch.tensor(_init(p, 37), device=cuda)
    a = f0.clone()
    ds.set_wait_limit(0)
    ds.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        ds.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
    ds.set_wait_limit(1 << 22)
    ds.step(a)
    ds.status()
    b = f0.clone()
    col.step(b)
    assert torch.equal(a, b)


def test_ds_slabs_autotune_keeps_the_bits(bkma, cuda):
    """The tuner picks among slabs per CTA and the column-pair kernels: the
    same bits whichever wins."""
    import torch
    p = AdvParams(*SLAB_CASES[0])
    ds, _, col = _slab_plans(bkma, p)
    f0 = torch.tensor(_init(p, 38), device=cuda)
    info = ds.autotune(f0.clone())
    assert info["path"] in (4, 5, 6), info
    a, b = f0.clone(), f0.clone()
    ds.step(a, nsteps=2)
    col.step(b, nsteps=2)
    assert torch.equal(a, b)


@pytest.mark.parametrize("R", [1, 2, 8, 16])
@pytest.mark.parametrize("degree", [5, 3])
def test_ds_runs_bit_identical_to_quads(bkma, cuda, R, degree):
    """The run-based kernel (W = 2: pairs of lines, or the two halves of one
    line per CTA; an odd last line pairs with itself) gives the 4-cell
    kernel's bits (W = 1)."""
    import torch
    p = AdvParams(21, 1024, 1, 0.0013, 0.0, 1.0, -2.0, 2.0)
    f0 = _init(p, 19)
    kw = dict(degree=degree, weights="reference" if degree == 5 else "lagrange")
    quad, _ = _rows_plans(bkma, p, **kw)
    quad.set_tile(1, 3, 256, 5)
    runs, _ = _rows_plans(bkma, p, **kw)
    assert runs.set_tile(2, R, 256, 5)["tile_cols"] == 2
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    quad.step(a, nsteps=3)
    runs.step(b, nsteps=3)
    runs.status()
    assert torch.equal(a, b)


@pytest.mark.parametrize("value", [1e200, float("inf")])
def test_ds_runs_unsplittable_value_runs_fp64(bkma, cuda, value):
    import torch
    p = AdvParams(4, 1024, 1, 0.003, 0.0, 1.0, -1.0, 1.0)
    ds, st = _rows_plans(bkma, p)
    ds.set_tile(2, 4, 256, 5)
    f0 = _init(p, 20)
    i0, r_bad = 2, 700
    f0[i0, r_bad, 0] = value
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    ds.step(a)
    st.step(b)
    ds.status()
    offs, _ = ds.line_table()
    rows = [r for r in range(p.n1) if (r_bad - (r + int(offs[i0]))) % p.n1 < 6]
    hit = torch.zeros_like(a, dtype=torch.bool)
    hit[i0, rows, 0] = True
    assert torch.allclose(a[hit], b[hit], rtol=0, atol=0, equal_nan=True)
    other = ~hit & torch.isfinite(b)
    assert (a - b)[other].abs().max().item() <= TOL * b[other].abs().max().item()


def test_ds_runs_exception_lines(bkma, cuda, oracle):
    """Pairs of lines where one or both are exception lines: the exception
    lines get the staged kernel's bits, their partners the pair arithmetic,
    the same bits as on the 4-cell kernel."""
    import torch
    p = AdvParams(6, 1000, 1, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    runs, st = _rows_plans(bkma, p, velocity=vel)
    runs.set_tile(2, 2, 256, 5)
    quad, _ = _rows_plans(bkma, p, velocity=vel)
    quad.set_tile(1, 3, 256, 5)
    f0 = _init(p, 29)
    a, b, c = (torch.tensor(f0, device=cuda) for _ in range(3))
    runs.step(a, nsteps=2)
    quad.step(b, nsteps=2)
    st.step(c, nsteps=2)
    runs.status()
    assert torch.equal(a, b)
    exc = [i0 for i0 in range(p.n0)
           if len({(oracle.departure(p, i1, vel[i0])[0] - i1) % p.n1 for i1 in range(p.n1)}) > 1]
    assert exc and len(exc) < p.n0
    for i0 in exc:
        assert torch.equal(a[i0], c[i0]), i0


def test_ds_runs_timeout_reported(bkma, cuda):
    import torch
    p = AdvParams(*ROWS_CASES[0])
    ds, _ = _rows_plans(bkma, p)
    ds.set_tile(2, 8, 256, 5)
    f0 = torch.tensor(_init(p, 30), device=cuda)
    a = f0.clone()
    ds.set_wait_limit(0)
    ds.step(a)
    with pytest.raises(bkma.BkmaError) as e:
        ds.status()
    assert e.value.status == 4
    assert torch.equal(a, f0)
