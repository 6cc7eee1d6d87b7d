"""Multi-process sharding of the advection path on CPU (gloo, world size 2).

Lines (i0, i2) are independent, so each rank advances its own slab range
(i0_offset / i0_count, as the C ABI takes them) with no exchange; gathering the
shards must reproduce the single-process run bit-for-bit. The per-rank compute
here is the oracle (no GPU on this machine); the GPU kernels get the same
offsets through bkma_adv_plan_create (tests/test_adv_gpu.py covers
sharded == full on the device)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n0, n1, n2, steps, result_q):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "parallel-advection_gb300"), os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    from bkma_gb300 import shard_lines
    from oracle import AdvParams, Oracle
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    orc = Oracle()
    p = AdvParams(n0=n0, n1=n1, n2=n2, dt=0.0015, minVx=-1.0, maxVx=1.0)
    rng = np.random.default_rng(7)
    full = rng.standard_normal((n0, n1, n2))
    off, cnt = shard_lines(n0, rank, world)
    mine = full[off:off + cnt].copy()  # a slice is a view: copy before stepping in place
    orc.adv_step(p, mine, steps, i0_offset=off, nthreads=1)
    # gather variable-size shards: pad to the largest
    maxc = -(-n0 // world)
    buf = torch.zeros((maxc, n1, n2), dtype=torch.float64)
    buf[:cnt] = torch.from_numpy(mine)
    bufs = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf)
    if rank == 0:
        parts = []
        for r in range(world):
            o, c = shard_lines(n0, r, world)
            parts.append(bufs[r][:c].numpy())
        gathered = np.concatenate(parts, 0)
        ref = orc.adv_step(p, full.copy(), steps, nthreads=1)
        result_q.put(bool(np.array_equal(gathered, ref)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("n0", [8, 7])
def test_two_rank_shards_equal_single_process(n0):
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n0, 64, 3, 3, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=120)
    assert all(pr.exitcode == 0 for pr in procs)
    assert q.get() is True


def test_shard_lines_partition():
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "parallel-advection_gb300"))
    from bkma_gb300 import shard_lines
    for n0 in (1, 2, 7, 2048, 2049):
        for world in (1, 2, 3, 8):
            if n0 < world:
                with pytest.raises(ValueError):
                    shard_lines(n0, 0, world)
                continue
            spans = [shard_lines(n0, r, world) for r in range(world)]
            assert spans[0][0] == 0
            assert sum(c for _, c in spans) == n0
            for (o1, c1), (o2, _) in zip(spans, spans[1:]):
                assert o1 + c1 == o2
