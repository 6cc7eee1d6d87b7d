"""BF16 tensor-core conv1d (tcgen05, FP32 accumulate in TMEM) against the
FP64 oracle evaluated on the same BF16-rounded inputs.

Tolerance: max |out - ref| <= 1e-2 * max |ref| (the BF16 output rounding alone
is 2^-9 relative); the tests also bound the mean error far tighter, at
3e-3 * max|ref|, to catch layout mistakes that only touch some elements.
Shapes run smallest first. In place (row stride L, a multiple of 8) the
epilogue stores through a TMA tensor map when cout >= 32 and L-K+1 >= 64;
out of place it does so only when L-K+1 is a multiple of 8, so the cases
below cover both epilogues, partial and empty last half-tiles and output
channel boxes clipped at cout.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [
    # B, C, L, K
    (1, 16, 256, 3),
    (1, 16, 136, 1),
    (1, 32, 136, 1),     # last tile: 8 positions, its second half-tile is empty
    (2, 32, 512, 7),
    (3, 64, 1000, 5),
    (2, 128, 1024, 7),
    (1, 128, 8192, 7),
    (2, 128, 1000, 9),   # taps 0-5 in TMEM (one accumulator), 6-8 in shared memory
    (2, 96, 512, 11),
]


def _case(shape, seed):
    B, C, L, K = shape
    rng = np.random.default_rng(seed)
    s = 1.0 / np.sqrt(C * K)
    x = rng.uniform(-1, 1, (B, C, L))
    w = rng.uniform(-1, 1, (C, C, K)) * s
    b = rng.uniform(-1, 1, C) * s
    return x, w, b


def _bf(cuda, a):
    import torch
    return torch.tensor(a, dtype=torch.float64, device=cuda).to(torch.bfloat16)


def _check(got, want):
    err = np.abs(got - want)
    scale = np.abs(want).max()
    assert err.max() <= 1e-2 * scale, (err.max(), scale)
    assert err.mean() <= 3e-3 * scale, (err.mean(), scale)


@pytest.mark.parametrize("shape", SHAPES)
def test_tensor_conv_inplace(bkma, cuda, oracle, shape):
    B, C, L, K = shape
    x, w, b = _case(shape, 100 + L)
    xd, wd, bd = _bf(cuda, x), _bf(cuda, w), _bf(cuda, b)
    want = oracle.conv_torch(xd.double().cpu().numpy(), wd.double().cpu().numpy(),
                             bd.double().cpu().numpy())
    orig = xd.clone()
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor")
    plan.run(xd, wd, bd)
    plan.status()
    got = xd.double().cpu().numpy()
    _check(got[:, :, :L - K + 1], want)
    # the tail keeps its input values
    assert np.array_equal(got[:, :, L - K + 1:], orig.double().cpu().numpy()[:, :, L - K + 1:])


@pytest.mark.parametrize("shape", [(2, 32, 512, 7), (2, 128, 1024, 7), (2, 128, 1032, 9),
                                   (2, 64, 520, 1)])
def test_tensor_conv_out_of_place_and_bias_none(bkma, cuda, oracle, shape):
    import torch
    B, C, L, K = shape
    x, w, _ = _case(shape, 7)
    xd, wd = _bf(cuda, x), _bf(cuda, w)
    want = oracle.conv_torch(xd.double().cpu().numpy(), wd.double().cpu().numpy(), None)
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor", inplace=False)
    out = torch.empty(B, C, L - K + 1, dtype=torch.bfloat16, device=cuda)
    before = xd.clone()
    plan.run(xd, wd, None, out=out)
    plan.status()
    _check(out.double().cpu().numpy(), want)
    assert torch.equal(xd, before)


@pytest.mark.parametrize("L,K", [(512, 3), (520, 9)])
def test_tensor_conv_fewer_out_channels(bkma, cuda, oracle, L, K):
    import torch
    B, cin, cout = 2, 64, 48
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (B, cin, L))
    w = rng.uniform(-1, 1, (cout, cin, K)) / np.sqrt(cin * K)
    b = rng.uniform(-1, 1, cout)
    xd, wd, bd = _bf(cuda, x), _bf(cuda, w), _bf(cuda, b)
    want = oracle.conv_torch(xd.double().cpu().numpy(), wd.double().cpu().numpy(),
                             bd.double().cpu().numpy())
    plan = bkma.Conv1dPlan(B, cin, cout, L, K, dtype="bf16", impl="tensor", inplace=False)
    out = torch.empty(B, cout, L - K + 1, dtype=torch.bfloat16, device=cuda)
    plan.run(xd, wd, bd, out=out)
    plan.status()
    _check(out.double().cpu().numpy(), want)


def test_tensor_conv_repeatable(bkma, cuda):
    """Two runs on the same input give identical bits (no race in the
    in-place halo handling)."""
    B, C, L, K = 4, 128, 4096, 7
    x, w, b = _case((B, C, L, K), 9)
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor")
    outs = []
    for _ in range(2):
        xd = _bf(cuda, x)
        plan.run(xd, _bf(cuda, w), _bf(cuda, b))
        plan.status()
        outs.append(xd)
    import torch
    assert torch.equal(outs[0], outs[1])


def test_tensor_conv_rejects_unsupported(bkma, cuda):
    with pytest.raises(bkma.BkmaError) as e:
        bkma.Conv1dPlan(2, 24, 24, 256, 3, dtype="bf16", impl="tensor")
    assert e.value.status == 2
    with pytest.raises(bkma.BkmaError):  # 7 taps of shared-memory weights leave no stages
        bkma.Conv1dPlan(2, 128, 128, 256, 13, dtype="bf16", impl="tensor")


@pytest.mark.parametrize("B", [640, 611])
def test_tensor_conv_chunk_rounds_against_torch(bkma, cuda, B):
    """Sizes with full rounds of 64-tile chunks over the CTAs plus an evenly
    split remainder (640 and 611 rows x 16 tiles), in place: every chunk
    boundary reads its halo from the snapshot. Reference: PyTorch's FP32
    conv1d on the same BF16 inputs (TF32 off)."""
    import torch
    C, L, K = 128, 2048, 7
    g = torch.Generator(device=cuda).manual_seed(B)
    s = 1.0 / (C * K) ** 0.5
    x = ((torch.rand((B, C, L), generator=g, device=cuda) * 2 - 1)).to(torch.bfloat16)
    w = ((torch.rand((C, C, K), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    b = ((torch.rand((C,), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    prev = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    try:
        want = torch.nn.functional.conv1d(x.float(), w.float(), b.float())
    finally:
        torch.backends.cudnn.allow_tf32 = prev
    orig_tail = x[:, :, L - K + 1:].clone()
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="bf16", impl="tensor")
    plan.run(x, w, b)
    plan.status()
    got = x[:, :, :L - K + 1].float()
    err = (got - want).abs()
    scale = want.abs().max()
    assert err.max() <= 1e-2 * scale, (err.max().item(), scale.item())
    assert err.mean() <= 3e-3 * scale, (err.mean().item(), scale.item())
    assert torch.equal(x[:, :, L - K + 1:], orig_tail)
