"""Parity at the benchmark workloads' full sizes, through properties that do
not need the oracle to run the whole field:

- advection 2048 x 1024 x 512 FP32, degree 5 (the bench workload: velocity
  law v_i = -1 + 2 i / (n0 - 1), dt = 1e-3): the default plan's
  kernel gives the bits of the generic staged kernel on the whole field;
  every line's sum over n1 is conserved (the incremental form
  f_c + sum_k w_k (f_k - f_c) conserves it exactly in exact arithmetic, for
  any weights); sampled slabs (the ends, the middle and random ones) are
  within the FP32 bound of the FP64 oracle;
- in-place BF16 conv1d B = 256, C = 128, L = 8192, K = 7: against PyTorch's
  FP32 conv1d (TF32 off) on the same BF16 inputs, and the last K - 1 samples
  of every row untouched;
- the 64-field uneven batch of the batched workload (about 4e9 cells): after
  the batch autotuner, every field has the bits of its own single plan;
- the advection workload's error target over its 50 steps, against the plain
  FP64 kernel (the reference's per-cell math, bit-exact with the oracle) from
  the same FP32-representable field: with the FP32 hi + lo state fused over
  the 50 steps (one FP32 rounding of the field), max |err| / max |f| <= 1e-6;
  one step per launch (FP32 rounding every step) within its documented
  bound, 8e-8 per step (8e-7 at 10 steps, 4e-6 at 50)."""
import numpy as np
import pytest

from oracle import AdvParams

pytestmark = pytest.mark.gpu

N0, N1, N2, DT, STEPS = 2048, 1024, 512, 1e-3, 2


def _release():
    import torch
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def test_advection_full_size(bkma, cuda, oracle):
    import torch
    vel = -1.0 + 2.0 * np.arange(N0, dtype=np.float64) / (N0 - 1)
    kw = dict(dtype="f32", degree=5, weights="reference", dt=DT, minX=0.0, maxX=1.0,
              minVx=-1.0, maxVx=1.0, velocity=vel)
    g = torch.Generator(device=cuda).manual_seed(12345)
    x = torch.arange(N1, device=cuda, dtype=torch.float32) / N1
    f0 = (torch.sin(2 * np.pi * x)[None, :, None]
          + 0.01 * (2 * torch.rand((N0, N1, N2), generator=g, device=cuda) - 1)).contiguous()
    rng = np.random.default_rng(7)
    slabs = sorted({0, 1, N0 // 2, N0 - 2, N0 - 1, *rng.integers(0, N0, 11).tolist()})
    init = f0[slabs].double().cpu().numpy()
    sums0 = torch.sum(f0, dim=1, dtype=torch.float64)

    plan = bkma.AdvectionPlan(N0, N1, N2, **kw)
    assert plan.info()["path"] in (1, 2), plan.info()  # TMA tiles or streamed columns
    a = f0.clone()
    plan.step(a, nsteps=STEPS)
    plan.status()
    staged = bkma.AdvectionPlan(N0, N1, N2, **kw)
    staged.set_tile(16, 1, 256, 0)
    staged.step(f0, nsteps=STEPS)
    staged.status()
    assert torch.equal(a, f0), "default kernel and generic staged kernel differ at full size"
    del f0

    # line sums: |sum_out - sum_in| within the FP32 rounding of n1 outputs
    # (each at most (npts + 2) roundings of values <= max|f|) per step
    drift = (torch.sum(a, dim=1, dtype=torch.float64) - sums0).abs().max().item()
    bound = STEPS * N1 * 8 * np.finfo(np.float32).eps * a.abs().max().item()
    assert drift <= bound, (drift, bound)

    p = AdvParams(N0, N1, N2, DT, 0.0, 1.0, -1.0, 1.0)
    got = a[slabs].double().cpu().numpy()
    for j, i0 in enumerate(slabs):
        want = oracle.adv_step(p, init[j:j + 1].copy(), STEPS, velocity=vel[i0:i0 + 1])
        err = np.abs(got[j:j + 1] - want).max() / np.abs(want).max()
        assert err <= 3e-7 * STEPS + 2e-7, (i0, err)
    del a, sums0
    _release()


def test_conv_full_size_inplace(bkma, cuda):
    import torch
    B, C, L, K = 256, 128, 8192, 7
    g = torch.Generator(device=cuda).manual_seed(2024)
    s = 1.0 / (C * K) ** 0.5
    x = ((torch.rand((B, C, L), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    w = ((torch.rand((C, C, K), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    b = ((torch.rand((C,), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    prev = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    try:
        want = torch.nn.functional.conv1d(x.float(), w.float(), b.float())
    finally:
        torch.backends.cudnn.allow_tf32 = prev
    tail = x[:, :, L - K + 1:].clone()
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor", inplace=True)
    plan.run(x, w, b)
    plan.status()
    assert torch.equal(x[:, :, L - K + 1:], tail)
    err = (x[:, :, :L - K + 1].float() - want).abs()
    scale = want.abs().max()
    assert err.max() <= 1e-2 * scale, (err.max().item(), scale.item())
    assert err.mean() <= 3e-3 * scale
    del x, want, err, tail
    _release()


def test_batched_full_size(bkma, cuda):
    import torch
    rng = np.random.default_rng(12345)
    g = torch.Generator(device=cuda).manual_seed(12345)
    fields, init = [], []
    for _ in range(64):
        n0 = int(rng.integers(64, 1025))
        n1 = int(rng.choice([256, 512, 1024, 2048]))
        n2 = int(rng.integers(1, 257))
        deg = int(rng.choice([3, 5]))
        x = torch.arange(n1, device=cuda, dtype=torch.float32) / n1
        d = (torch.sin(2 * np.pi * x)[None, :, None]
             + 0.01 * (2 * torch.rand((n0, n1, n2), generator=g, device=cuda) - 1)).contiguous()
        fields.append(dict(data=d, degree=deg, weights="reference" if deg == 5 else "lagrange",
                           dt=DT, minX=0.0, maxX=1.0, minVx=-2.0, maxVx=2.0,
                           velocity=rng.uniform(-2.0, 2.0, n0)))
        init.append(d.clone())
    batch = bkma.AdvectionBatch(fields, dtype="f32")
    assert batch.cells > 2e9
    batch.autotune()
    for f, d0 in zip(fields, init):  # the autotuner steps the fields: restart
        f["data"].copy_(d0)
    batch.step(STEPS)
    torch.cuda.synchronize()
    for f, d0 in zip(fields, init):
        n0, n1, n2 = d0.shape
        kw = {k: f[k] for k in ("degree", "weights", "dt", "minX", "maxX", "minVx", "maxVx",
                                "velocity")}
        bkma.AdvectionPlan(n0, n1, n2, dtype="f32", **kw).step(d0, nsteps=STEPS)
        assert torch.equal(f["data"], d0), (n0, n1, n2, f["degree"])
    del fields, init, batch
    _release()


def test_advection_50_step_error_targets(bkma, cuda):
    import torch
    vel = -1.0 + 2.0 * np.arange(N0, dtype=np.float64) / (N0 - 1)
    kw = dict(dt=DT, minX=0.0, maxX=1.0, minVx=-1.0, maxVx=1.0, velocity=vel)
    plain = bkma.AdvectionPlan(N0, N1, N2, dtype="f64", impl="plain", **kw)
    ref = torch.empty((N0, N1, N2), dtype=torch.float64, device=cuda)
    plain.fill(ref, mode=1, amp=0.01, seed=12345)
    f0 = ref.float()
    ref.copy_(f0)
    ref10 = ref.clone()
    plain.step(ref10, nsteps=10)
    plain.step(ref, nsteps=50)
    plain.status()

    one = bkma.AdvectionPlan(N0, N1, N2, dtype="f32", **kw)
    fused = bkma.AdvectionPlan(N0, N1, N2, dtype="f32", **kw)
    fused.set_fused_state("f32x2")
    fused.set_fusion(50)
    x = f0.clone()
    fused.step(x, nsteps=50)
    fused.status()
    nx = one.error_norms(x, ref)
    assert nx["max_rel"] <= 1e-6, nx
    assert nx["l2_rel"] <= 1e-7, nx

    x.copy_(f0)
    one.step(x, nsteps=10)
    n10 = one.error_norms(x, ref10)
    assert n10["max_rel"] <= 8e-8 * 10, n10
    one.step(x, nsteps=40)
    one.status()
    n50 = one.error_norms(x, ref)
    assert n50["max_rel"] <= 8e-8 * 50, n50
    assert n50["l2_rel"] <= 1e-6, n50
    del ref, ref10, f0, x
    _release()
