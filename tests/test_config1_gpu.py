"""The CPU-runnable advection workload at its stated parameters, on the GPU:
FP64 n0 = 512 velocity lines x n1 = 1024 periodic cells x n2 = 1, line
velocities v_i = -1 + 2 i / 511 (passed as a per-line velocity array),
dx = 1/1024 on [0, 1), dt = 0.001, degree 5 (the reference's stencil), init
sin(2 pi x) + U[-0.01, 0.01] from numpy's default_rng(12345), 10 steps.

- the plain FP64 kernel (the reference's per-cell math) is bit-exact with the
  oracle after every step;
- the FP64 default (contiguous lines in FP32-pair arithmetic) and the staged
  FP64 kernel are within 1e-11 max|f| of it (per-line weights);
- the FP32 kernels are within the FP32 storage bound.

A second case runs the reference's own law (v_i = minVx + i (maxVx - minVx) /
n0, src/config/AdvectionParams.cpp:100) with its init sin(4 pi x)
(src/tools/init.hpp:43) and its analytic check (src/tools/validation.hpp:9-80).
"""
import numpy as np
import pytest

from oracle import AdvParams

pytestmark = pytest.mark.gpu

N0, N1, N2, DT, STEPS, SEED = 512, 1024, 1, 0.001, 10, 12345


def _params():
    return AdvParams(N0, N1, N2, DT, 0.0, 1.0, -1.0, 1.0)


def _velocity():
    return -1.0 + 2.0 * np.arange(N0, dtype=np.float64) / (N0 - 1)


def _init():
    rng = np.random.default_rng(SEED)
    x = np.arange(N1) / N1
    return np.ascontiguousarray(np.sin(2 * np.pi * x)[None, :, None]
                                + 0.01 * rng.uniform(-1, 1, (N0, N1, N2)))


def _plan(bkma, **kw):
    return bkma.AdvectionPlan(N0, N1, N2, dt=DT, minX=0.0, maxX=1.0, minVx=-1.0, maxVx=1.0,
                              velocity=_velocity(), **kw)


def test_config1_plain_fp64_bitexact_every_step(bkma, cuda, oracle):
    import torch
    p, vel = _params(), _velocity()
    f0 = _init()
    want = f0.copy()
    plan = _plan(bkma, dtype="f64", impl="plain")
    d = torch.tensor(f0, dtype=torch.float64, device=cuda)
    for step in range(1, STEPS + 1):
        plan.step(d)
        oracle.adv_step(p, want, 1, velocity=vel)
        assert np.array_equal(d.cpu().numpy(), want), f"step {step}"


@pytest.mark.parametrize("path", [None, 0])  # the default (FP32-pair contiguous lines), FP64 staged
def test_config1_staged_fp64(bkma, cuda, oracle, path):
    import torch
    p, vel = _params(), _velocity()
    f0 = _init()
    want = oracle.adv_step(p, f0.copy(), STEPS, velocity=vel)
    plan = _plan(bkma, dtype="f64")
    if path is None:
        assert plan.info()["path"] == 5, plan.info()
    else:
        plan.set_tile(1, 8, 256, path)
    d = torch.tensor(f0, dtype=torch.float64, device=cuda)
    plan.step(d, nsteps=STEPS)
    plan.status()
    err = np.abs(d.cpu().numpy() - want).max() / np.abs(want).max()
    assert err <= 1e-11, err


@pytest.mark.parametrize("path", [None, 0])  # the default (contiguous lines) and generic staged tiles
def test_config1_fp32(bkma, cuda, oracle, path):
    import torch
    p, vel = _params(), _velocity()
    f0 = _init().astype(np.float32).astype(np.float64)
    want = oracle.adv_step(p, f0.copy(), STEPS, velocity=vel)
    plan = _plan(bkma, dtype="f32")
    if path is not None:
        plan.set_tile(1, 8, 256, path)
    d = torch.tensor(f0, dtype=torch.float32, device=cuda)
    plan.step(d, nsteps=STEPS)
    plan.status()
    err = np.abs(d.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
    assert err <= 8e-8 * STEPS, err


def test_config1_reference_law_and_init(bkma, cuda, oracle):
    """The reference's velocity law and sin(4 pi x) init: the device fill
    within 2 ulp of the oracle's (libm sin), plain FP64 steps bit-exact with
    the oracle from the same field, the device analytic check equal to the
    oracle's and below the reference tests' 1e-6
    (tests/validation_unittests.cpp:34-94)."""
    import torch
    p = _params()
    plan = bkma.AdvectionPlan(N0, N1, N2, dtype="f64", impl="plain", dt=DT, minX=0.0,
                              maxX=1.0, minVx=-1.0, maxVx=1.0)
    d = torch.empty((N0, N1, N2), dtype=torch.float64, device=cuda)
    plan.fill(d, mode=0)
    # the device sin and the host's libm sin may differ in the last bit
    fill = oracle.fill_adv(p)
    assert np.abs(d.cpu().numpy() - fill).max() <= 2 * np.finfo(np.float64).eps
    ref = d.cpu().numpy().copy()
    plan.step(d, nsteps=STEPS)
    oracle.adv_step(p, ref, STEPS)
    assert np.array_equal(d.cpu().numpy(), ref)
    hi, _ = plan.validate(d, STEPS)
    assert hi < 1e-6
    assert abs(hi - oracle.validate_adv(p, ref, STEPS)) <= 1e-12
