"""Learned stencils on the GPU (bkma_mlp_*), against the FP64 oracle
(oracle/mlp_oracle.py, itself checked against torch autograd): the 4-point
model on the config's fine lines (n1 = 1024, degree-9 targets), and the
6-point model on under-resolved lines (n1 = 128, 32 modes, exact targets),
where it beats the degree-5 stencil it corrects.

Tolerances: generator |diff| <= 2e-6 (FP32 line values), inference <= 2e-6,
gradient relative L2 <= 1e-4 and loss relative <= 1e-4 (FP32 forward and
gradient sums against FP64)."""
import numpy as np
import pytest

import mlp_oracle as M
from oracle import AdvParams

pytestmark = pytest.mark.gpu


def test_generator_matches_oracle(bkma, cuda):
    a, f4, t = bkma.LearnedStencil.samples(3000, 21, first=5)
    oa, of4, ot = M.make_samples(3000, 21, first=5)
    assert np.abs(a.cpu().numpy() - oa).max() <= 1e-7
    assert np.abs(f4.cpu().numpy() - of4).max() <= 2e-6
    assert np.abs(t.cpu().numpy() - ot).max() <= 2e-6


def test_init_and_inference_match_oracle(bkma, cuda):
    import torch
    net = bkma.LearnedStencil(seed=4)
    p = net.params().astype(np.float64)
    assert np.abs(p - M.init_params(4)).max() <= 1e-7
    rng = np.random.default_rng(1)
    q = M.init_params(4)
    q[M.OFF_W3:] = 0.05 * rng.standard_normal(M.NP - M.OFF_W3)
    q = q.astype(np.float32)
    net.set_params(q)
    alpha = np.linspace(0, 1, 257, endpoint=False)
    w = net.infer(torch.tensor(alpha, dtype=torch.float32, device=cuda)).cpu().numpy()
    want = M.weights(q.astype(np.float64), alpha.astype(np.float32).astype(np.float64))
    assert np.abs(w - want).max() <= 2e-6
    assert np.abs(w.sum(1) - 1.0).max() <= 1e-6


def test_gradient_matches_oracle(bkma, cuda):
    net = bkma.LearnedStencil(seed=8)
    rng = np.random.default_rng(2)
    q = M.init_params(8)
    q[M.OFF_W3:] = 0.05 * rng.standard_normal(M.NP - M.OFF_W3)
    q = q.astype(np.float32)
    net.set_params(q)
    a, f4, t = bkma.LearnedStencil.samples(640, 33)
    loss, g = net.grad(a, f4, t)
    ol, og = M.loss_and_grad(q.astype(np.float64), a.double().cpu().numpy(),
                             f4.double().cpu().numpy(), t.double().cpu().numpy())
    assert abs(loss - ol) <= 1e-4 * ol
    assert np.linalg.norm(g - og) <= 1e-4 * np.linalg.norm(og)


def test_training_beats_lagrange3_on_held_out_lines(bkma, cuda):
    import torch
    net = bkma.LearnedStencil(seed=3)
    a, f4, t = bkma.LearnedStencil.samples(1 << 17, 5)
    net.train(a, f4, t, steps=800, batch=4096, lr=3e-3)
    va, vf, vt = bkma.LearnedStencil.samples(1 << 15, 5, first=1 << 24)
    w = net.infer(va)
    learned = float(((w * vf).sum(1) - vt).double().pow(2).mean())
    l3 = torch.tensor(M.lagrange(4, 1.0 + va.double().cpu().numpy()), device=cuda)
    base = float(((l3 * vf.double()).sum(1) - vt.double()).pow(2).mean())
    assert learned < 0.5 * base, (learned, base)


def test_learned_advection_beats_lagrange3(bkma, cuda):
    """20 advection steps of a band-limited periodic field: the learned 4-point
    stencil is closer to the exact shifted solution than degree-3 Lagrange."""
    import torch
    net = bkma.LearnedStencil(seed=3)
    a, f4, t = bkma.LearnedStencil.samples(1 << 17, 5)
    net.train(a, f4, t, steps=800, batch=4096, lr=3e-3)
    p = AdvParams(16, 1024, 4, 0.0007, 0.0, 1.0, -1.0, 1.0)
    rng = np.random.default_rng(9)
    modes = np.arange(1, 33)
    am = rng.uniform(-1, 1, modes.size) / modes
    bm = rng.uniform(-1, 1, modes.size) / modes

    def f(x):
        ph = 2 * np.pi * np.outer(x, modes)
        return (np.cos(ph) * am + np.sin(ph) * bm).sum(1)

    x = np.arange(p.n1) / p.n1
    f0 = np.repeat(f(x)[None, :, None], p.n0, 0).repeat(p.n2, 2)
    steps = 20
    kw = dict(dt=p.dt, minX=0.0, maxX=1.0, minVx=-1.0, maxVx=1.0)
    learned = net.plan_for(p.n0, p.n1, p.n2, **kw)
    lag3 = bkma.AdvectionPlan(p.n0, p.n1, p.n2, dtype="f32", degree=3, weights="lagrange", **kw)
    errs = {}
    for name, plan in (("learned", learned), ("lagrange3", lag3)):
        d = torch.tensor(f0, dtype=torch.float32, device=cuda)
        plan.step(d, nsteps=steps)
        got = d.double().cpu().numpy()
        err = 0.0
        for i0 in range(p.n0):
            v = -1.0 + i0 * (2.0 / p.n0)
            exact = f((x - v * steps * p.dt) % 1.0)
            err += ((got[i0, :, 0] - exact) ** 2).mean()
        errs[name] = err / p.n0
    assert errs["learned"] < errs["lagrange3"], errs


# under-resolved lines: 32 modes on 128 cells (half the grid's Nyquist band)
COARSE = dict(n1=128, npts=6, exact=True)


def test_six_point_generator_matches_oracle(bkma, cuda):
    a, f, t = bkma.LearnedStencil.samples(3000, 21, first=5, **COARSE)
    oa, of, ot = M.make_samples(3000, 21, first=5, **COARSE)
    assert f.shape == (3000, 6)
    assert np.abs(a.cpu().numpy() - oa).max() <= 1e-7
    assert np.abs(f.cpu().numpy() - of).max() <= 2e-6
    assert np.abs(t.cpu().numpy() - ot).max() <= 2e-6


def test_six_point_inference_and_gradient_match_oracle(bkma, cuda):
    import torch
    net = bkma.LearnedStencil(seed=4, npts=6)
    assert net.npts == 6 and net.NP == M.nparams(6) == 1318
    p = net.params().astype(np.float64)
    assert np.abs(p - M.init_params(4, 6)).max() <= 1e-7
    rng = np.random.default_rng(1)
    q = M.init_params(4, 6)
    q[M.OFF_W3:] = 0.05 * rng.standard_normal(M.nparams(6) - M.OFF_W3)
    q = q.astype(np.float32)
    net.set_params(q)
    alpha = np.linspace(0, 1, 257, endpoint=False)
    w = net.infer(torch.tensor(alpha, dtype=torch.float32, device=cuda)).cpu().numpy()
    want = M.weights(q.astype(np.float64), alpha.astype(np.float32).astype(np.float64), 6)
    assert np.abs(w - want).max() <= 2e-6
    assert np.abs(w.sum(1) - 1.0).max() <= 1e-6
    a, f, t = bkma.LearnedStencil.samples(640, 33, **COARSE)
    loss, g = net.grad(a, f, t)
    ol, og = M.loss_and_grad(q.astype(np.float64), a.double().cpu().numpy(),
                             f.double().cpu().numpy(), t.double().cpu().numpy())
    assert abs(loss - ol) <= 1e-4 * ol
    assert np.linalg.norm(g - og) <= 1e-4 * np.linalg.norm(og)


def _trained_six_point(bkma):
    net = bkma.LearnedStencil(seed=3, npts=6)
    a, f, t = bkma.LearnedStencil.samples(1 << 18, 5, **COARSE)
    net.train(a, f, t, steps=2000, batch=8192, lr=3e-3)
    return net


def test_six_point_beats_degree5_on_under_resolved_lines(bkma, cuda):
    import torch
    net = _trained_six_point(bkma)
    va, vf, vt = bkma.LearnedStencil.samples(1 << 15, 5, first=1 << 24, **COARSE)
    w = net.infer(va)
    learned = float(((w * vf).sum(1) - vt).double().pow(2).mean())
    l5 = torch.tensor(M.lagrange(6, 2.0 + va.double().cpu().numpy()), device=cuda)
    base = float(((l5 * vf.double()).sum(1) - vt.double()).pow(2).mean())
    assert learned < 0.25 * base, (learned, base)


def test_six_point_advection_beats_degree5(bkma, cuda):
    """30 advection steps of a 32-mode periodic field on 128-cell lines: the
    learned 6-point stencil ends closer to the exact shifted solution than
    the reference's degree-5 stencil and textbook degree-5 Lagrange, with the
    same taps and the same kernel."""
    import torch
    net = _trained_six_point(bkma)
    p = AdvParams(16, 128, 4, 0.003, 0.0, 1.0, -1.0, 1.0)
    rng = np.random.default_rng(9)
    modes = np.arange(1, 33)
    am = rng.uniform(-1, 1, modes.size) / modes
    bm = rng.uniform(-1, 1, modes.size) / modes

    def f(x):
        ph = 2 * np.pi * np.outer(x, modes)
        return (np.cos(ph) * am + np.sin(ph) * bm).sum(1)

    x = np.arange(p.n1) / p.n1
    f0 = np.repeat(f(x)[None, :, None], p.n0, 0).repeat(p.n2, 2)
    steps = 30
    kw = dict(dt=p.dt, minX=0.0, maxX=1.0, minVx=-1.0, maxVx=1.0)
    plans = {"learned6": net.plan_for(p.n0, p.n1, p.n2, **kw),
             "degree5_reference": bkma.AdvectionPlan(p.n0, p.n1, p.n2, dtype="f32", **kw),
             "degree5_lagrange": bkma.AdvectionPlan(p.n0, p.n1, p.n2, dtype="f32", degree=5,
                                                    weights="lagrange", **kw)}
    errs = {}
    for name, plan in plans.items():
        d = torch.tensor(f0, dtype=torch.float32, device=cuda)
        plan.step(d, nsteps=steps)
        got = d.double().cpu().numpy()
        err = 0.0
        for i0 in range(p.n0):
            v = -1.0 + i0 * (2.0 / p.n0)
            exact = f((x - v * steps * p.dt) % 1.0)
            err += ((got[i0, :, 0] - exact) ** 2).mean()
        errs[name] = err / p.n0
    assert errs["learned6"] < 0.5 * min(errs["degree5_reference"], errs["degree5_lagrange"]), errs
