"""FP64 advection in FP32-pair arithmetic, streamed down column pairs (path 6),
through the C ABI.

The streamed form computes every cell with the same operations as the staged
column-pair kernel (path 4), so the two give the same bits wherever both
apply, walking up the rows or, for lines shifted npts + 2 or more rows down,
down them; it is the default for column pairs the staged form cannot take
(lines too tall for a shared-memory strip, rows 1 MB or more apart). Tolerances as
in test_adv_ds_gpu.py: 2e-13 max|f| per step against the FP64 staged kernel,
1e-11 against the oracle; windows the FP32 pair cannot carry, exception lines
and fields off the 16-byte grid run the staged kernel's FP64 arithmetic.
"""
import numpy as np
import pytest

from oracle import AdvParams

pytestmark = pytest.mark.gpu

TOL = 2e-13
CASES = [
    # n0, n1, n2, dt, minX, maxX, minVx, maxVx
    (4, 1024, 64, 0.001, 0.0, 1.0, -1.0, 1.0),
    (3, 256, 130, 0.003, 0.0, 1.0, -2.0, 2.0),    # groups spanning two lines
    (5, 300, 38, 0.005, 0.0, 1.0, -3.0, 3.0),     # shifts of several cells, n1 % 12 != 0
    (2, 2048, 96, 0.0007, -0.5, 1.5, -1.0, 1.0),
]


def _init(p, seed):
    rng = np.random.default_rng(seed)
    x = p.minX + np.arange(p.n1) * ((p.maxX - p.minX) / p.n1)
    f = np.sin(2 * np.pi * (x - p.minX) / (p.maxX - p.minX))[None, :, None]
    return np.ascontiguousarray(f + 0.01 * rng.uniform(-1, 1, (p.n0, p.n1, p.n2)))


def _plan(bkma, p, **kw):
    args = dict(dt=p.dt, minX=p.minX, maxX=p.maxX, minVx=p.minVx, maxVx=p.maxVx, dtype="f64")
    args.update(kw)
    return bkma.AdvectionPlan(p.n0, p.n1, p.n2, **args)


def _staged(bkma, p, **kw):
    st = _plan(bkma, p, **kw)
    st.set_tile(1, 1, 256, 0)
    return st


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("degree", [5, 3])
def test_stream_ds_equals_column_pair_kernel(bkma, cuda, oracle, case, degree):
    import torch
    p = AdvParams(*case)
    weights = "reference" if degree == 5 else "lagrange"
    s6 = _plan(bkma, p, degree=degree, weights=weights)
    s6.set_tile(8, 0, 256, 6)
    s4 = _plan(bkma, p, degree=degree, weights=weights)
    s4.set_tile(4, 1, 128, 4)
    st = _staged(bkma, p, degree=degree, weights=weights)
    f0 = _init(p, 21)
    steps = 3
    a, b, c = (torch.tensor(f0, device=cuda) for _ in range(3))
    s6.step(a, nsteps=steps)
    s4.step(b, nsteps=steps)
    st.step(c, nsteps=steps)
    s6.status()
    assert torch.equal(a, b)
    assert (a - c).abs().max().item() <= TOL * steps * c.abs().max().item()
    want = oracle.adv_step(p, f0.copy(), steps, degree=degree, ref_weights=degree == 5)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


@pytest.mark.parametrize("segs", [1, 2, 4, 8])
def test_stream_ds_row_segments_bit_identical(bkma, cuda, segs):
    """Rows split between warps (seams in shared memory) give the same bits."""
    import torch
    p = AdvParams(*CASES[0])
    ref = _plan(bkma, p)
    ref.set_tile(8, 1, 256, 6)
    seg = _plan(bkma, p)
    seg.set_tile(8, segs, 256, 6)
    f0 = _init(p, 22)
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    ref.step(a, nsteps=3)
    seg.step(b, nsteps=3)
    seg.status()
    assert torch.equal(a, b)


def test_stream_ds_tall_lines_default(bkma, cuda, oracle):
    """Lines too tall for a shared-memory strip of 4 FP64 columns stream."""
    import torch
    p = AdvParams(2, 16384, 8, 0.001, 0.0, 1.0, -1.0, 1.0)
    plan = _plan(bkma, p)
    assert plan.info()["path"] == 6, plan.info()
    f0 = _init(p, 23)
    a = torch.tensor(f0, device=cuda)
    plan.step(a, nsteps=2)
    plan.status()
    want = oracle.adv_step(p, f0.copy(), 2)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_stream_ds_far_rows_default(bkma, cuda):
    """Rows 1 MB or more apart stream; the result equals the column-pair kernel."""
    import torch
    p = AdvParams(1, 128, 131072, 0.002, 0.0, 1.0, -1.0, 1.0)
    plan = _plan(bkma, p)
    assert plan.info()["path"] == 6, plan.info()
    s4 = _plan(bkma, p)
    s4.set_tile(4, 1, 128, 4)
    f0 = _init(p, 24)
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    plan.step(a, nsteps=2)
    s4.step(b, nsteps=2)
    plan.status()
    assert torch.equal(a, b)


def test_stream_ds_inplace_equals_out_of_place(bkma, cuda):
    import torch
    p = AdvParams(*CASES[1])
    ip = _plan(bkma, p)
    ip.set_tile(8, 0, 256, 6)
    oop = _plan(bkma, p, inplace=False)
    oop.set_tile(8, 0, 256, 6)
    f0 = _init(p, 25)
    a = torch.tensor(f0, device=cuda)
    ip.step(a, nsteps=3)
    src = torch.tensor(f0, device=cuda)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(a, out)


@pytest.mark.parametrize("value", [1e200, 1e-30, float("inf")])
def test_stream_ds_unsplittable_value_runs_fp64(bkma, cuda, value):
    import torch
    p = AdvParams(3, 256, 24, 0.003, 0.0, 1.0, -1.0, 1.0)
    s6 = _plan(bkma, p)
    s6.set_tile(8, 0, 256, 6)
    s4 = _plan(bkma, p)
    s4.set_tile(4, 1, 128, 4)
    f0 = _init(p, 26)
    f0[1, 100, 11] = value
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    s6.step(a)
    s4.step(b)
    s6.status()
    # both forms send the same windows to the FP64 arithmetic
    assert torch.allclose(a, b, rtol=0, atol=0, equal_nan=True)


def test_stream_ds_exception_lines_bit_identical_to_staged(bkma, cuda, oracle):
    import torch
    p = AdvParams(6, 1000, 8, 0.001, 0.0, 1.0, -2.0, 3.0)
    vel = np.array([1.0, 0.37, -2.0, 0.5, 3.0, -0.77])
    s6 = _plan(bkma, p, velocity=vel)
    s6.set_tile(8, 0, 256, 6)
    assert s6.info()["exception_lines"] > 0
    s4 = _plan(bkma, p, velocity=vel)
    s4.set_tile(4, 1, 128, 4)
    f0 = _init(p, 27)
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    s6.step(a, nsteps=2)
    s4.step(b, nsteps=2)
    s6.status()
    assert torch.equal(a, b)


def test_stream_ds_misaligned_field_runs_fp64(bkma, cuda):
    import torch
    p = AdvParams(*CASES[0])
    s6 = _plan(bkma, p)
    s6.set_tile(8, 0, 256, 6)
    st = _staged(bkma, p)
    f0 = _init(p, 28)
    buf = torch.empty(f0.size + 1, dtype=torch.float64, device=cuda)
    d = buf[1:].view(f0.shape)  # 8 bytes past a 16-byte boundary
    d.copy_(torch.tensor(f0, device=cuda))
    s6.step(d, nsteps=2)
    b = torch.tensor(f0, device=cuda)
    st.step(b, nsteps=2)
    assert torch.equal(d, b)


# per-line velocities whose shifts run from -12.6 to +26.6 cells (n1 = 1024,
# dt = 0.001): tap-0 offsets d from about +10 down to -29; each 64-column group
# is one line (n2 = 64), and the lines with d <= -(npts + 2) walk down their rows
FAR_VEL = np.array([-12.3, -6.0, 0.3, 5.0, 9.0, 13.0, 20.0, 26.0])


@pytest.mark.parametrize("degree", [5, 3])
def test_stream_ds_large_shifts_walk_down(bkma, cuda, oracle, degree):
    """Lines shifted 12 or more rows down stream walking down their rows: the
    same bits as the column-pair kernel, in place as out of place."""
    import torch
    p = AdvParams(8, 1024, 64, 0.001, 0.0, 1.0, -1.0, 1.0)
    weights = "reference" if degree == 5 else "lagrange"
    kw = dict(velocity=FAR_VEL, degree=degree, weights=weights)
    s6 = _plan(bkma, p, **kw)
    s6.set_tile(8, 0, 256, 6)
    s4 = _plan(bkma, p, **kw)
    s4.set_tile(4, 1, 128, 4)
    oop = _plan(bkma, p, inplace=False, **kw)
    oop.set_tile(8, 0, 256, 6)
    f0 = _init(p, 29)
    a, b, src = (torch.tensor(f0, device=cuda) for _ in range(3))
    s6.step(a, nsteps=3)
    s4.step(b, nsteps=3)
    s6.status()
    assert torch.equal(a, b)
    out = torch.empty_like(src)
    oop.step(src, out=out, nsteps=3)
    assert torch.equal(a, out)
    want = oracle.adv_step(p, f0.copy(), 3, degree=degree, ref_weights=degree == 5,
                           velocity=FAR_VEL)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_stream_ds_group_votes_one_direction(bkma, cuda):
    """A 64-column group spanning 8 lines (n2 = 8) whose shifts straddle the
    up/down limit walks down as a whole: the column-pair kernel's bits."""
    import torch
    p = AdvParams(16, 512, 8, 0.002, 0.0, 1.0, -1.0, 1.0)
    vel = np.linspace(2.0, 14.0, 16)  # shifts 2.0 .. 14.3 cells
    s6 = _plan(bkma, p, velocity=vel)
    s6.set_tile(8, 0, 256, 6)
    s4 = _plan(bkma, p, velocity=vel)
    s4.set_tile(4, 1, 128, 4)
    f0 = _init(p, 30)
    a, b = torch.tensor(f0, device=cuda), torch.tensor(f0, device=cuda)
    s6.step(a, nsteps=2)
    s4.step(b, nsteps=2)
    s6.status()
    assert torch.equal(a, b)


def test_stream_ds_refuses_groups_with_no_direction(bkma, cuda):
    """Lines 12 rows down and 12 rows up in one group (n2 = 2: 32 lines per
    group) suit neither walk: the plan keeps the staged kernels."""
    p = AdvParams(64, 1024, 2, 0.001, 0.0, 1.0, -1.0, 1.0)
    vel = np.where(np.arange(64) % 2 == 0, 14.0, -14.0)
    plan = _plan(bkma, p, velocity=vel)
    assert plan.info()["path"] != 6
    with pytest.raises(bkma.BkmaError):
        plan.set_tile(8, 0, 256, 6)


def test_stream_ds_long_lines_large_shifts_default(bkma, cuda, oracle):
    """The reference's 1024 x 16384 x 128 sweep shape shifts lines by up to 16
    cells per step (16384 cells, dt = 0.001, v in [-1, 1]): its slabs stream,
    the last of these four walking down (shifts -16.4, -4.9, 6.6, 16.4)."""
    import torch
    p = AdvParams(4, 16384, 128, 0.001, 0.0, 1.0, -1.0, 1.0)
    vel = np.array([-1.0, -0.3, 0.4, 1.0])
    plan = _plan(bkma, p, velocity=vel)
    assert plan.info()["path"] == 6, plan.info()
    f0 = _init(p, 31)
    a = torch.tensor(f0, device=cuda)
    plan.step(a, nsteps=2)
    plan.status()
    want = oracle.adv_step(p, f0.copy(), 2, velocity=vel)
    assert np.abs(a.cpu().numpy() - want).max() <= 1e-11 * np.abs(want).max()


def test_stream_ds_zero_field_stays_zero(bkma, cuda):
    import torch
    p = AdvParams(*CASES[0])
    s6 = _plan(bkma, p)
    s6.set_tile(8, 0, 256, 6)
    z = torch.zeros((p.n0, p.n1, p.n2), dtype=torch.float64, device=cuda)
    s6.step(z, nsteps=3)
    assert torch.count_nonzero(z).item() == 0
