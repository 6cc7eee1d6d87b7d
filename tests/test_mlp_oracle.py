"""The learned-stencil oracle (oracle/mlp_oracle.py) itself: its hand-written
backward pass against torch autograd in float64 (4- and 6-point models), the
untrained model being exactly the Lagrange stencil of its degree, and a
reproducible sample generator (degree-9 and exact targets). CPU only."""
import numpy as np
import pytest
import torch

import mlp_oracle as M


def _torch_loss(p, a, f, t):
    npts = f.shape[1]
    ob3 = M.off_b3(npts)
    pt = torch.tensor(p, requires_grad=True)
    W1, b1 = pt[M.OFF_W1:M.OFF_B1], pt[M.OFF_B1:M.OFF_W2]
    W2, b2 = pt[M.OFF_W2:M.OFF_B2].view(32, 32), pt[M.OFF_B2:M.OFF_W3]
    W3, b3 = pt[M.OFF_W3:ob3].view(npts, 32), pt[ob3:ob3 + npts]
    at = torch.tensor(a)[:, None]
    h1 = torch.nn.functional.gelu(at * W1 + b1)
    h2 = torch.nn.functional.gelu(h1 @ W2.T + b2)
    c = h2 @ W3.T + b3
    w = torch.tensor(M.lagrange(npts, npts // 2 - 1 + a)) + c - c.mean(1, keepdim=True)
    loss = ((w * torch.tensor(f)).sum(1) - torch.tensor(t)).pow(2).mean()
    loss.backward()
    return loss.item(), pt.grad.numpy()


@pytest.mark.parametrize("npts,n1,exact", [(4, 1024, False), (6, 128, True)])
def test_backward_matches_torch_autograd(npts, n1, exact):
    rng = np.random.default_rng(0)
    p = M.init_params(3, npts)
    p[M.OFF_W3:] = 0.05 * rng.standard_normal(M.nparams(npts) - M.OFF_W3)
    a, f, t = M.make_samples(300, 11, n1=n1, npts=npts, exact=exact)
    assert f.shape == (300, npts)
    loss, g = M.loss_and_grad(p, a, f, t)
    tl, tg = _torch_loss(p, a, f, t)
    assert abs(loss - tl) <= 1e-14 * max(1.0, tl)
    assert np.abs(g - tg).max() <= 1e-12 * np.abs(tg).max()


def test_untrained_six_point_model_is_lagrange5():
    p = M.init_params(5, 6)
    assert p.size == 1318
    a = np.linspace(0, 1, 17, endpoint=False)
    assert np.array_equal(M.weights(p, a, 6), M.lagrange(6, 2.0 + a))


def test_exact_targets():
    """On fine lines the degree-9 target and the line's exact value agree;
    on 128-cell lines (32 modes: half of the grid's Nyquist band) degree 9 is
    off, and degree 5 far more than on fine lines."""
    a, f, t9 = M.make_samples(2000, 4, n1=1024, npts=6)
    _, _, te = M.make_samples(2000, 4, n1=1024, npts=6, exact=True)
    assert np.abs(t9 - te).max() < 1e-9
    a, f, t9 = M.make_samples(2000, 4, n1=128, npts=6)
    _, _, te = M.make_samples(2000, 4, n1=128, npts=6, exact=True)
    assert np.abs(t9 - te).max() > 1e-6
    l5 = (M.lagrange(6, 2.0 + a) * f).sum(1)
    assert ((l5 - te) ** 2).mean() > 1e-7


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
