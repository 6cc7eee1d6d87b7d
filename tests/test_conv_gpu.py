"""Conv1d parity on the GPU through the C ABI.

Tolerances:
  - REFERENCE semantics (ConvSolver + AdaptiveWg packing), FP64: bit-exact
    against the oracle and the reference's golden vectors;
  - TORCH semantics, FP64 plain kernel: bit-exact against the oracle (same
    bias / ci / k accumulation order, no contraction);
  - TORCH semantics, FP32 plain kernel: |err| <= 1e-5 * max|out| against FP64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(cuda, a, dtype=None):
    import torch
    return torch.tensor(a, dtype=dtype or torch.float64, device=cuda)


@pytest.mark.parametrize("name", ["rand", "wide"])
def test_reference_semantics_golden(bkma, cuda, golden, name):
    n0, C, L, n2, K = (int(v) for v in golden[f"conv_{name}_meta"])
    plan = bkma.Conv1dPlan(n0, C, C, L, K, dtype="f64", semantics="reference", n2=n2)
    d = _t(cuda, golden[f"conv_{name}_in"])
    plan.run(d, _t(cuda, golden[f"conv_{name}_w"]), _t(cuda, golden[f"conv_{name}_b"]))
    assert np.array_equal(d.cpu().numpy(), golden[f"conv_{name}_out"])


@pytest.mark.parametrize("shape", [(2, 3, 16, 1, 3), (3, 5, 33, 7, 4), (1, 2, 200, 40, 11)])
def test_reference_semantics_oracle(bkma, cuda, oracle, shape):
    import torch
    n0, C, L, n2, K = shape
    rng = np.random.default_rng(sum(shape))
    data = rng.standard_normal((n0, C * L, n2))
    w = rng.standard_normal((K, C, C))
    b = rng.standard_normal(C)
    plan = bkma.Conv1dPlan(n0, C, C, L, K, dtype="f64", semantics="reference", n2=n2)
    d = _t(cuda, data)
    plan.run(d, _t(cuda, w), _t(cuda, b))
    want = oracle.conv_ref_step(data.copy(), w, b, K, C, L)
    assert np.array_equal(d.cpu().numpy(), want)
    # out of place leaves the input alone and gives the same output
    src = _t(cuda, data)
    out = torch.empty_like(src)
    plan.run(src, _t(cuda, w), _t(cuda, b), out=out)
    assert np.array_equal(out.cpu().numpy(), want)
    assert np.array_equal(src.cpu().numpy(), data)


@pytest.mark.parametrize("shape", [(2, 4, 4, 64, 3), (3, 6, 6, 130, 7), (2, 16, 16, 257, 5),
                                   (1, 3, 5, 20, 20)])
@pytest.mark.parametrize("inplace", [True, False])
def test_torch_semantics_fp64_bitexact(bkma, cuda, oracle, shape, inplace):
    import torch
    B, cin, cout, L, K = shape
    if inplace and cin != cout:
        pytest.skip("in place needs cin == cout")
    rng = np.random.default_rng(L)
    x = rng.standard_normal((B, cin, L))
    w = rng.standard_normal((cout, cin, K))
    b = rng.standard_normal(cout)
    plan = bkma.Conv1dPlan(B, cin, cout, L, K, dtype="f64", impl="plain", inplace=inplace)
    want = oracle.conv_torch(x, w, b)
    d = _t(cuda, x)
    if inplace:
        plan.run(d, _t(cuda, w), _t(cuda, b))
        got = d.cpu().numpy()
        assert np.array_equal(got[:, :, :L - K + 1], want)
        assert np.array_equal(got[:, :, L - K + 1:], x[:, :, L - K + 1:])
    else:
        out = torch.empty(B, cout, L - K + 1, dtype=torch.float64, device=cuda)
        plan.run(d, _t(cuda, w), _t(cuda, b), out=out)
        assert np.array_equal(out.cpu().numpy(), want)


def test_torch_semantics_fp32(bkma, cuda, oracle):
    import torch
    B, C, L, K = 4, 32, 300, 7
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, (B, C, L)).astype(np.float32)
    w = (rng.uniform(-1, 1, (C, C, K)) / np.sqrt(C * K)).astype(np.float32)
    b = rng.uniform(-1, 1, C).astype(np.float32)
    plan = bkma.Conv1dPlan(B, C, C, L, K, dtype="f32", impl="plain")
    d = _t(cuda, x, torch.float32)
    plan.run(d, _t(cuda, w, torch.float32), _t(cuda, b, torch.float32))
    want = oracle.conv_torch(x.astype(np.float64), w.astype(np.float64), b.astype(np.float64))
    got = d.cpu().numpy()[:, :, :L - K + 1].astype(np.float64)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_halo_scratch_is_reported(bkma, cuda):
    plan = bkma.Conv1dPlan(2, 8, 8, 512, 7, dtype="f32", impl="plain")
    assert plan.scratch_bytes() == 4 * 2 * ((512 - 7 + 1 + 63) // 64) * 8 * 6


@pytest.mark.parametrize("dtype", ["f32", "f64", "bf16"])
def test_device_fill_and_conv_check(bkma, cuda, dtype):
    """fill_buffer_conv1d and the conv1d checks (validation.hpp:84-156) on
    the device: a constant field is all-equal with the constant as mean; a
    changed value breaks equality; the mean of random data equals numpy's
    over the first nw values of every line."""
    import torch
    tdt = {"f32": torch.float32, "f64": torch.float64, "bf16": torch.bfloat16}[dtype]
    n0, n1, n2, nw = 5, 300, 7, 250
    d = torch.empty((n0, n1, n2), dtype=tdt, device=cuda)
    bkma.fill(d, 7.3)
    want = float(torch.tensor(7.3, dtype=tdt))
    assert torch.equal(d, torch.full_like(d, 7.3))
    mean, equal = bkma.conv_check(d, nw)
    assert equal and abs(mean - want) <= 1e-12 * abs(want)
    d[3, nw - 1, 6] = 1.0
    assert not bkma.conv_check(d, nw)[1]
    assert bkma.conv_check(d, nw - 1)[1]   # the changed value lies beyond nw - 1
    d[3, 0, 0] = float("nan")
    assert not bkma.conv_check(d, 1)[1]
    r = torch.rand((n0, n1, n2), dtype=torch.float64, device=cuda).to(tdt)
    mean, equal = bkma.conv_check(r, nw)
    ref = r[:, :nw, :].double().cpu().numpy().mean()
    assert not equal and abs(mean - ref) <= 1e-12
    one = torch.full((1, 4, 1), float("nan"), dtype=tdt, device=cuda)
    assert bkma.conv_check(one, 4)[1]  # nothing to compare, as in the reference
