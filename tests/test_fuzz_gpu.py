"""Seeded random shapes through the default plans.

Advection: each plan's own kernel choice (TMA tiles, streamed columns,
contiguous lines, staged whole rows) against the generic staged kernel on
the same field: identical bits after three steps, in place; fields small
enough for the oracle also stay within the FP32 bound of the FP64 oracle;
degree-5 FP64 plans stay within 1e-11 max|f| of the plain FP64 form.
Conv1d (tensor path, BF16): random batch, channels, length and kernel size
against PyTorch's FP32 conv1d on the same BF16 inputs (TF32 off), in place
and out of place."""
import numpy as np
import pytest

from oracle import AdvParams

pytestmark = pytest.mark.gpu


def _adv_cases(n=24, seed=2026):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        n1 = int(rng.choice([16, 20, 64, 100, 256, 333, 1024, 2048, 3000]))
        n2 = int(rng.choice([1, 1, 2, 3, 4, 7, 8, 13, 16, 32, 37, 64, 100]))
        n0 = int(rng.integers(1, max(2, min(64, 400000 // (n1 * n2)) + 1)))
        deg = int(rng.choice([3, 5, 9]))
        vmax = float(rng.choice([0.5, 1.0, 3.0, 20.0]))
        dt = float(rng.choice([1e-4, 1e-3, 4e-3]))
        out.append((n0, n1, n2, deg, vmax, dt))
    return out


@pytest.mark.parametrize("case", _adv_cases())
def test_fuzz_advection_paths_agree(bkma, cuda, oracle, case):
    import torch
    n0, n1, n2, deg, vmax, dt = case
    p = AdvParams(n0, n1, n2, dt, 0.0, 1.0, -vmax, vmax)
    kw = dict(dtype="f32", degree=deg, weights="reference" if deg == 5 else "lagrange",
              dt=dt, minX=0.0, maxX=1.0, minVx=-vmax, maxVx=vmax)
    rng = np.random.default_rng(n0 * 7919 + n1 * 31 + n2)
    x = np.arange(n1) / n1
    f0 = (np.sin(2 * np.pi * x)[None, :, None]
          + 0.01 * rng.uniform(-1, 1, (n0, n1, n2))).astype(np.float32)
    auto = bkma.AdvectionPlan(n0, n1, n2, **kw)
    staged = bkma.AdvectionPlan(n0, n1, n2, **kw)
    staged.set_tile(min(16, n2), 1, 256, 0)
    a = torch.tensor(f0, device=cuda)
    s = torch.tensor(f0, device=cuda)
    auto.step(a, nsteps=3)
    staged.step(s, nsteps=3)
    auto.status()
    staged.status()
    assert torch.equal(a, s), auto.info()
    if n0 * n1 * n2 <= 200000:
        want = oracle.adv_step(p, f0.astype(np.float64), 3, degree=deg, ref_weights=deg == 5)
        err = np.abs(a.cpu().numpy().astype(np.float64) - want).max() / np.abs(want).max()
        assert err <= 3e-7 * 3 + 2e-7 + (1e-6 if deg == 9 else 0.0), (err, auto.info())
    if deg == 5:
        # FP64: the default plan (direct stencil sum) against the plain form
        # (the reference's per-cell arithmetic, bit-exact with the oracle)
        kw64 = dict(kw, dtype="f64")
        d = torch.tensor(f0.astype(np.float64), device=cuda)
        r = d.clone()
        bkma.AdvectionPlan(n0, n1, n2, **kw64).step(d, nsteps=3)
        bkma.AdvectionPlan(n0, n1, n2, impl="plain", **kw64).step(r, nsteps=3)
        assert ((d - r).abs().max() <= 1e-11 * r.abs().max()).item()


def _conv_cases(n=10, seed=77):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        c = int(rng.choice([16, 32, 48, 64, 96, 128]))
        k = int(rng.integers(1, 10))
        length = int(8 * rng.integers(max(2, (k + 7) // 8 + 1), 400))
        b = int(rng.integers(1, 9))
        out.append((b, c, length, k, bool(rng.integers(0, 2))))
    return out


@pytest.mark.parametrize("case", _conv_cases())
def test_fuzz_tensor_conv_against_torch(bkma, cuda, case):
    import torch
    B, C, L, K, inplace = case
    g = torch.Generator(device=cuda).manual_seed(B * 1000 + C * 10 + K)
    s = 1.0 / (C * K) ** 0.5
    x = (torch.rand((B, C, L), generator=g, device=cuda) * 2 - 1).to(torch.bfloat16)
    w = ((torch.rand((C, C, K), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    b = ((torch.rand((C,), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    prev = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    try:
        want = torch.nn.functional.conv1d(x.float(), w.float(), b.float())
    finally:
        torch.backends.cudnn.allow_tf32 = prev
    try:
        plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor", inplace=inplace)
    except bkma.BkmaError as e:  # shapes the tensor path does not take
        assert e.status == 2
        pytest.skip(str(e))
    if inplace:
        tail = x[:, :, L - K + 1:].clone()
        plan.run(x, w, b)
        plan.status()
        got = x[:, :, :L - K + 1].float()
        assert torch.equal(x[:, :, L - K + 1:], tail)
    else:
        out = torch.empty((B, C, L - K + 1), dtype=torch.bfloat16, device=cuda)
        plan.run(x, w, b, out=out)
        plan.status()
        got = out.float()
    err = (got - want).abs()
    scale = want.abs().max()
    assert err.max() <= 1e-2 * scale, (err.max().item(), scale.item())
    assert err.mean() <= 3e-3 * scale


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_fuzz_batch_equals_single_plans(bkma, cuda, seed):
    """A random uneven batch (streamed, staged and exception-line fields of
    degree 3 and 5, n2 from 1 up) gives, after the batch autotuner, the bits
    of every field advanced alone by its own plan."""
    import torch
    rng = np.random.default_rng(seed)
    fields, singles = [], []
    for _ in range(int(rng.integers(3, 9))):
        n0 = int(rng.integers(1, 40))
        n1 = int(rng.choice([64, 100, 256, 512, 1024, 2048]))
        n2 = int(rng.integers(1, 80))
        deg = int(rng.choice([3, 5]))
        vel = rng.uniform(-3.0, 3.0, n0)
        if rng.integers(0, 3) == 0:  # a few lines with shifts of whole cells
            vel[: max(1, n0 // 4)] = np.round(vel[: max(1, n0 // 4)])
        f0 = (rng.uniform(-1, 1, (n0, n1, n2))).astype(np.float32)
        kw = dict(degree=deg, weights="reference" if deg == 5 else "lagrange", dt=1.0 / n1,
                  minX=0.0, maxX=1.0, minVx=-3.0, maxVx=3.0, velocity=vel)
        fields.append(dict(data=torch.tensor(f0, device=cuda), **kw))
        singles.append((torch.tensor(f0, device=cuda), kw))
    batch = bkma.AdvectionBatch(fields, dtype="f32")
    batch.autotune()
    for f, (s, _) in zip(fields, singles):  # the autotuner steps the fields: reset
        f["data"].copy_(s)
    batch.step(3)
    torch.cuda.synchronize()
    for f, (s, kw) in zip(fields, singles):
        n0, n1, n2 = s.shape
        bkma.AdvectionPlan(n0, n1, n2, dtype="f32", **kw).step(s, nsteps=3)
        assert torch.equal(f["data"], s)


@pytest.mark.parametrize("case", _adv_cases(n=8, seed=4040))
def test_fuzz_fused_steps(bkma, cuda, case):
    """Random shapes: k fused steps per launch give the bits of one step per
    launch, and the hi + lo state at one step per launch gives the FP32 bits."""
    import torch
    n0, n1, n2, deg, vmax, dt = case
    kw = dict(dtype="f32", degree=deg, weights="reference" if deg == 5 else "lagrange",
              dt=dt, minX=0.0, maxX=1.0, minVx=-vmax, maxVx=vmax)
    rng = np.random.default_rng(n0 + n1 + n2)
    f0 = rng.uniform(-1, 1, (n0, n1, n2)).astype(np.float32)
    ref = torch.tensor(f0, device=cuda)
    bkma.AdvectionPlan(n0, n1, n2, **kw).step(ref, nsteps=5)
    fz = bkma.AdvectionPlan(n0, n1, n2, **kw)
    try:
        fz.set_fusion(3)
    except bkma.BkmaError:  # lines the fused strips cannot hold
        pytest.skip("no fused strip for this shape")
    d = torch.tensor(f0, device=cuda)
    fz.step(d, nsteps=5)
    fz.status()
    assert torch.equal(d, ref)
    x2 = bkma.AdvectionPlan(n0, n1, n2, **kw)
    try:
        x2.set_fused_state("f32x2")
    except bkma.BkmaError:
        return
    x2.set_fusion(2)
    e = torch.tensor(f0, device=cuda)
    for _ in range(5):
        x2.step(e, nsteps=1)
    assert torch.equal(e, ref)


def _pair_cases(n=16, seed=909):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        if rng.integers(0, 2):
            n1 = int(rng.choice([16, 20, 64, 100, 256, 300, 1000, 1024, 2048, 4096, 8192, 16384]))
            n2 = 1
        else:
            n1 = int(rng.choice([12, 16, 40, 64, 100, 127, 128, 256, 1000]))
            n2 = int(rng.choice([2, 4, 6, 8, 10, 24, 64, 130]))
        n0 = int(rng.integers(1, max(2, min(24, 600000 // (n1 * n2)) + 1)))
        deg = int(rng.choice([3, 5]))
        vmax = float(rng.choice([0.5, 2.0, 8.0]))
        dt = float(rng.choice([1e-4, 1e-3, 3e-3]))
        out.append((n0, n1, n2, deg, vmax, dt, int(rng.integers(0, 1 << 30))))
    # the long-line forms (half lines from 8192 cells, runs of 4-cell groups)
    # and large shifts on streamed column pairs, whatever the draws gave
    out += [(3, 16384, 1, 5, 2.0, 1e-3, 11), (2, 8192, 1, 3, 8.0, 3e-3, 12),
            (4, 4096, 1, 5, 2.0, 1e-3, 13), (6, 64, 130, 5, 2.0, 1e-3, 14),
            (5, 1024, 8, 5, 8.0, 3e-3, 15), (4, 2048, 64, 3, 3.0, 2e-3, 16)]
    return out


@pytest.mark.parametrize("case", _pair_cases())
def test_fuzz_fp64_pair_forms_agree(bkma, cuda, case):
    """Random FP64 shapes: every FP32-pair form the plan accepts (contiguous
    lines: 4-cell groups, runs along two sections, half lines in clusters,
    runs of 4-cell groups, any lines per CTA; even n2: whole slabs with any
    runs per column pair, staged and streamed column pairs) gives the same
    bits, lines shifted by whole cells (exception lines) included, and the
    default plan stays within 1e-11 of the plain FP64 form (degree 5), or
    2e-13 per step of the FP64-arithmetic staged kernel (degree 3)."""
    import torch
    n0, n1, n2, deg, vmax, dt, seed = case
    rng = np.random.default_rng(seed)
    vel = rng.uniform(-vmax, vmax, n0)
    vel[:: 3] = np.round(vel[:: 3] * dt * n1) / (dt * n1)  # whole-cell shifts
    kw = dict(dtype="f64", degree=deg, weights="reference" if deg == 5 else "lagrange", dt=dt,
              minX=0.0, maxX=1.0, minVx=-vmax, maxVx=vmax, velocity=vel)
    x = np.arange(n1) / n1
    f0 = np.sin(2 * np.pi * x)[None, :, None] + 0.01 * rng.uniform(-1, 1, (n0, n1, n2))
    if n2 == 1:
        forms = [(W, R, 256, 5) for W in (1, 2, 3, 4, 5, 6) for R in (1, 2, 3, 8)]
    else:
        forms = ([(W, R, 256, 5) for W in (1, 2, 4) for R in (1, 3)]
                 + [(4, 1, 128, 4), (8, 1, 256, 4), (8, 0, 256, 6), (8, 2, 256, 6)])
    outs = []
    for tile in forms:
        plan = bkma.AdvectionPlan(n0, n1, n2, **kw)
        try:
            plan.set_tile(*tile)
        except bkma.BkmaError:
            continue  # not a form this shape takes
        d = torch.tensor(f0, device=cuda)
        plan.step(d, nsteps=2)
        plan.status()
        outs.append((tile, d))
    if outs:
        ref_tile, ref = outs[0]
        for tile, d in outs[1:]:
            assert torch.equal(d, ref), (ref_tile, tile)
    auto = bkma.AdvectionPlan(n0, n1, n2, **kw)
    d = torch.tensor(f0, device=cuda)
    auto.step(d, nsteps=2)
    auto.status()
    r = torch.tensor(f0, device=cuda)
    if deg == 5:
        # the plain form: the reference's per-cell arithmetic
        bkma.AdvectionPlan(n0, n1, n2, impl="plain", **kw).step(r, nsteps=2)
        tol = 1e-11
    else:
        # the FP64-arithmetic staged kernel, same weights: 2e-13 per step
        st = bkma.AdvectionPlan(n0, n1, n2, **kw)
        st.set_tile(1, 1, 256, 0)
        st.step(r, nsteps=2)
        tol = 4e-13
    assert ((d - r).abs().max() <= tol * r.abs().max()).item(), auto.info()
