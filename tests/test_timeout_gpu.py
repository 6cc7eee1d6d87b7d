"""Device-side timeout reporting, exercised without a stuck GPU.

The kernels with device-side waits (the TMA-staged and contiguous-line
advection kernels and the tensor-core conv1d pipeline) bound every wait and report a timeout through a
status word that the plan's status call returns as BKMA_ERR_TIMEOUT (the
reference raises C++ exceptions instead, src/core/bkma_tools.hpp:38-51). A
plan's wait limit set to 0 makes every wait give up at once: the launch stops
without writing its tiles, waits for its own copies and MMAs in flight, frees
its tensor memory, and the context stays usable. These tests check the whole
path: the status is reported once, then cleared, and the next call with the
default limit gives the normal result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEFAULT_POLLS = 1 << 22


def _field(cuda, shape, seed):
    import torch
    g = torch.Generator(device=cuda).manual_seed(seed)
    x = torch.arange(shape[1], device=cuda, dtype=torch.float32) / shape[1]
    return (torch.sin(2 * np.pi * x)[None, :, None]
            + 0.01 * (2 * torch.rand(shape, generator=g, device=cuda) - 1)).contiguous()


def test_adv_tma_timeout_reported_then_cleared(bkma, cuda):
    import torch
    shape = (4, 512, 32)
    kw = dict(dtype="f32", dt=1e-3, minX=0.0, maxX=1.0, minVx=-1.0, maxVx=1.0)
    plan = bkma.AdvectionPlan(*shape, **kw)
    assert plan.info()["path"] == 1, plan.info()  # TMA-staged tiles
    f0 = _field(cuda, shape, 3)
    d = f0.clone()
    plan.set_wait_limit(0)
    plan.step(d)
    with pytest.raises(bkma.BkmaError) as e:
        plan.status()
    assert e.value.status == 4  # BKMA_ERR_TIMEOUT
    assert "timed out" in str(e.value)
    plan.status()  # cleared by the previous query
    # no tile was written: every CTA gave up before its stores
    assert torch.equal(d, f0)
    # the context is usable and the default limit gives the normal bits
    plan.set_wait_limit(DEFAULT_POLLS)
    plan.step(d)
    plan.status()
    fresh = bkma.AdvectionPlan(*shape, **kw)
    want = f0.clone()
    fresh.step(want)
    fresh.status()
    assert torch.equal(d, want)


def test_adv_rows_timeout_reported_then_cleared(bkma, cuda):
    """The contiguous-line kernel (n2 = 1) stages its lines with one bulk copy
    completed on an mbarrier: its bounded wait reports the same way."""
    import torch
    shape = (64, 256, 1)
    kw = dict(dtype="f32", dt=1e-3, minX=0.0, maxX=1.0, minVx=-1.0, maxVx=1.0)
    plan = bkma.AdvectionPlan(*shape, **kw)
    assert plan.info()["path"] == 3, plan.info()  # runs of contiguous lines
    f0 = _field(cuda, shape, 5)
    d = f0.clone()
    plan.set_wait_limit(0)
    plan.step(d)
    with pytest.raises(bkma.BkmaError) as e:
        plan.status()
    assert e.value.status == 4  # BKMA_ERR_TIMEOUT
    plan.status()  # cleared
    assert torch.equal(d, f0)  # no CTA wrote its lines
    plan.set_wait_limit(DEFAULT_POLLS)
    plan.step(d)
    plan.status()
    fresh = bkma.AdvectionPlan(*shape, **kw)
    want = f0.clone()
    fresh.step(want)
    fresh.status()
    assert torch.equal(d, want)


def test_conv_tc_timeout_reported_then_cleared(bkma, cuda):
    import torch
    B, C, L, K = 2, 64, 1024, 5
    g = torch.Generator(device=cuda).manual_seed(11)
    s = 1.0 / (C * K) ** 0.5
    x0 = ((torch.rand((B, C, L), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    w = ((torch.rand((C, C, K), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    b = ((torch.rand((C,), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor")
    x = x0.clone()
    plan.set_wait_limit(0)
    plan.run(x, w, b)
    with pytest.raises(bkma.BkmaError) as e:
        plan.status()
    assert e.value.status == 4  # BKMA_ERR_TIMEOUT
    plan.status()  # cleared
    assert torch.equal(x, x0)  # the pipeline stopped before any output store
    plan.set_wait_limit(DEFAULT_POLLS)
    plan.run(x, w, b)
    plan.status()
    want = x0.clone()
    fresh = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor")
    fresh.run(want, w, b)
    fresh.status()
    assert torch.equal(x, want)


def test_plain_paths_have_no_waits(bkma, cuda):
    """Kernels without device-side waits ignore the limit: the status stays OK."""
    import torch
    shape = (4, 2048, 16)  # streamed columns
    plan = bkma.AdvectionPlan(*shape, dtype="f32", dt=1e-3, minX=0.0, maxX=1.0,
                              minVx=-1.0, maxVx=1.0)
    assert plan.info()["path"] == 2
    d = _field(cuda, shape, 5)
    plan.set_wait_limit(0)
    plan.step(d)
    plan.status()
    assert torch.isfinite(d).all()
