"""The learned-stencil oracle (oracle/mlp_oracle.py) itself: its hand-written
backward pass against torch autograd in float64, the untrained model being
exactly degree-3 Lagrange, and a reproducible sample generator. CPU only."""
import numpy as np
import torch

import mlp_oracle as M


def _torch_loss(p, a, f4, t):
    pt = torch.tensor(p, requires_grad=True)
    W1, b1 = pt[M.OFF_W1:M.OFF_B1], pt[M.OFF_B1:M.OFF_W2]
    W2, b2 = pt[M.OFF_W2:M.OFF_B2].view(32, 32), pt[M.OFF_B2:M.OFF_W3]
    W3, b3 = pt[M.OFF_W3:M.OFF_B3].view(4, 32), pt[M.OFF_B3:M.NP]
    at = torch.tensor(a)[:, None]
    h1 = torch.nn.functional.gelu(at * W1 + b1)
    h2 = torch.nn.functional.gelu(h1 @ W2.T + b2)
    c = h2 @ W3.T + b3
    w = torch.tensor(M.lagrange(4, 1.0 + a)) + c - c.mean(1, keepdim=True)
    loss = ((w * torch.tensor(f4)).sum(1) - torch.tensor(t)).pow(2).mean()
    loss.backward()
    return loss.item(), pt.grad.numpy()


def test_backward_matches_torch_autograd():
    rng = np.random.default_rng(0)
    p = M.init_params(3)
    p[M.OFF_W3:] = 0.05 * rng.standard_normal(M.NP - M.OFF_W3)
    a, f4, t = M.make_samples(300, 11)
    loss, g = M.loss_and_grad(p, a, f4, t)
    tl, tg = _torch_loss(p, a, f4, t)
    assert abs(loss - tl) <= 1e-14 * max(1.0, tl)
    assert np.abs(g - tg).max() <= 1e-12 * np.abs(tg).max()


def test_untrained_model_is_lagrange3():
    p = M.init_params(5)
    a = np.linspace(0, 1, 17, endpoint=False)
    assert np.array_equal(M.weights(p, a), M.lagrange(4, 1.0 + a))


def test_samples_reproducible_and_sliceable():
    a1, f1, t1 = M.make_samples(50, 9)
    a2, f2, t2 = M.make_samples(20, 9, first=30)
    assert np.array_equal(a1[30:], a2) and np.array_equal(f1[30:], f2) and np.array_equal(t1[30:], t2)
    assert (a1 >= 0).all() and (a1 < 1).all()
    # the degree-9 target is far closer to the 4-point data than a bad guess
    l3 = (M.lagrange(4, 1.0 + a1) * f1).sum(1)
    assert np.abs(l3 - t1).max() < 1e-3
