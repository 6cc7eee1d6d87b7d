"""The allocation-free conv1d entry point, called through the C ABI.

bkma_conv1d_bf16_inplace_noalloc serves callers that must not allocate device
memory while they run (runtimes that own the whole device heap, loops that
cannot afford an allocation's implicit synchronization); it keeps its scratch
in a fixed device array inside the library. This file is collected last so
that a run stopping at the first failure has already run every other test.

Its output must equal the plan-based entry point's (bkma_conv_run): the same
kernels run in the same order, so the check is exact; the tensor-path
tolerance of the other tests (1e-2 * max|ref| against FP64) is also asserted.
Two calls in a row use different inputs, so a stale scratch array would show.
"""
import ctypes as C
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(cuda, seed, B, Ch, L, K):
    import torch
    g = torch.Generator(device=cuda).manual_seed(seed)
    s = 1.0 / (Ch * K) ** 0.5
    x = ((torch.rand((B, Ch, L), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    w = ((torch.rand((Ch, Ch, K), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    b = ((torch.rand((Ch,), generator=g, device=cuda) * 2 - 1) * s).to(torch.bfloat16)
    return x, w, b


def _noalloc(lib, x, w, b, stream):
    B, Ch, L = x.shape
    K = w.shape[2]
    return lib.bkma_conv1d_bf16_inplace_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()),
                                                C.c_void_p(b.data_ptr()), B, Ch, L, K,
                                                C.c_void_p(stream))


def test_noalloc_matches_plan_entry_point_twice(bkma, cuda, oracle):
    import torch
    lib = bkma.load()
    stream = torch.cuda.current_stream().cuda_stream
    shapes = [(2, 128, 1024, 7), (3, 64, 2048, 5)]
    for call, (B, Ch, L, K) in enumerate(shapes):
        x, w, b = _inputs(cuda, 100 + call, B, Ch, L, K)
        want = x.clone()
        plan = bkma.Conv1dPlan(B, Ch, Ch, L, K, dtype="bf16", impl="tensor")
        plan.run(want, w, b)
        plan.status()
        got = x.clone()
        assert _noalloc(lib, got, w, b, stream) == 0, lib.bkma_last_error().decode()
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call}: differs from bkma_conv_run"
        ref = oracle.conv_torch(x.double().cpu().numpy(), w.double().cpu().numpy(),
                                b.double().cpu().numpy())
        err = np.abs(got.double().cpu().numpy()[:, :, :L - K + 1] - ref).max()
        assert err <= 1e-2 * np.abs(ref).max()


def test_noalloc_allocates_nothing(bkma, cuda):
    """After the first call (which looks the array's address up and loads the
    kernels), repeated calls change neither the device's free memory nor the
    torch allocator's counters, and the status call reports each call OK."""
    import torch
    lib = bkma.load()
    stream = torch.cuda.current_stream().cuda_stream
    B, Ch, L, K = 4, 128, 2048, 7
    x, w, b = _inputs(cuda, 21, B, Ch, L, K)
    assert _noalloc(lib, x.clone(), w, b, stream) == 0, lib.bkma_last_error().decode()
    assert lib.bkma_conv1d_noalloc_status(C.c_void_p(stream)) == 0
    bufs = [x.clone() for _ in range(3)]
    gc.collect()  # earlier tests' leftovers must not be freed inside the window
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for buf in bufs:
        assert _noalloc(lib, buf, w, b, stream) == 0, lib.bkma_last_error().decode()
        assert lib.bkma_conv1d_noalloc_status(C.c_void_p(stream)) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0, (free0, free1)
    # cumulative counts of allocator requests and of device segments it reserved
    for k in ("allocation.all.allocated", "segment.all.allocated"):
        assert stats1.get(k, 0) == stats0.get(k, 0), k
    assert torch.equal(bufs[0], bufs[1]) and torch.equal(bufs[1], bufs[2])


def test_noalloc_refuses_out_of_bounds_arguments(bkma, cuda):
    """The same argument bounds as the plan entry point: a huge ksize is refused
    before anything runs, not truncated to a small one."""
    import torch
    lib = bkma.load()
    stream = torch.cuda.current_stream().cuda_stream
    x, w, b = _inputs(cuda, 5, 1, 16, 8192, 3)
    got = lib.bkma_conv1d_bf16_inplace_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()),
                                               C.c_void_p(b.data_ptr()), 1, 16, 8192,
                                               (1 << 32) + 3, C.c_void_p(stream))
    assert got == 1, got  # BKMA_ERR_INVALID_ARG
    got = lib.bkma_conv1d_bf16_inplace_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()),
                                               C.c_void_p(b.data_ptr()), 1, 16, 8192, 5000,
                                               C.c_void_p(stream))
    assert got == 1, got


def test_noalloc_large_batch_matches_plan(bkma, cuda):
    """The halo snapshot keeps one slot per chunk of tiles, so a batch whose per-tile
    snapshot would not have fit the fixed array (160 rows x 64 tiles x 128
    channels x 16 bytes = 21 MB > 15.5 MiB) runs and equals bkma_conv_run."""
    import torch
    lib = bkma.load()
    stream = torch.cuda.current_stream().cuda_stream
    B, Ch, L, K = 160, 128, 8192, 7
    x, w, b = _inputs(cuda, 7, B, Ch, L, K)
    want = x.clone()
    plan = bkma.Conv1dPlan(B, Ch, Ch, L, K, dtype="bf16", impl="tensor")
    plan.run(want, w, b)
    plan.status()
    assert _noalloc(lib, x, w, b, stream) == 0, lib.bkma_last_error().decode()
    torch.cuda.synchronize()
    assert torch.equal(x, want)


def test_noalloc_replays_in_a_cuda_graph(bkma, cuda):
    """After one call outside a capture (it resolves the fixed array's
    address), the entry point records into a CUDA graph on a side stream:
    replays over new inputs written into the same buffers equal bkma_conv_run,
    and a replay allocates nothing."""
    import torch
    lib = bkma.load()
    B, Ch, L, K = 4, 128, 4096, 7
    x, w, b = _inputs(cuda, 11, B, Ch, L, K)
    assert _noalloc(lib, x.clone(), w, b, torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        rc = _noalloc(lib, x, w, b, side.cuda_stream)
    assert rc == 0, lib.bkma_last_error().decode()
    plan = bkma.Conv1dPlan(B, Ch, Ch, L, K, dtype="bf16", impl="tensor")
    for seed in (12, 13):
        x2, w2, b2 = _inputs(cuda, seed, B, Ch, L, K)
        want = x2.clone()
        plan.run(want, w2, b2)
        plan.status()
        x.copy_(x2)
        w.copy_(w2)
        b.copy_(b2)
        torch.cuda.synchronize()
        mem0 = torch.cuda.memory_allocated()
        g.replay()
        torch.cuda.synchronize()
        assert torch.cuda.memory_allocated() == mem0
        assert lib.bkma_conv1d_noalloc_status(C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        assert torch.equal(x, want), seed
