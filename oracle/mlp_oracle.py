"""CPU oracle of the learned stencils (FP64 numpy). TEST INFRASTRUCTURE ONLY:
the checker for csrc/mlp.cu's data generator, forward, backward and
inference kernels.

Model (same layout as the CUDA kernels), npts = 4 or 6 stencil points:
  params (32 + 32 + 1024 + 32 + 33 npts floats: 1252 for 4 points, 1318 for 6)
       = [W1 (32) | b1 (32) | W2 (32x32, [out][in]) | b2 (32) |
          W3 (npts x 32, [out][in]) | b3 (npts)]
  h1 = gelu(W1 * a + b1); h2 = gelu(W2 h1 + b2); c = W3 h2 + b3
  w(a) = lagrange_{npts}(npts/2 - 1 + a) + c - mean(c)  (the weights sum to 1)
  prediction = sum_k w_k * f[k], f = the npts nodes from j - (npts/2 - 1)
  loss = mean over the batch of (prediction - target)^2
gelu(x) = x/2 (1 + erf(x/sqrt 2)).

Training samples: a random periodic line f(x) = sum_{m=1..M} a_m cos(2 pi m x)
+ b_m sin(2 pi m x), a_m, b_m ~ U[-1, 1]/m, 10 nodes x_k = x0 + (k-4)/n1
(k = 0..9), a shift a; the target is the degree-9 Lagrange interpolation of
the 10 nodes at 4 + a, or (exact) f(x0 + a/n1). Random numbers come from the
counter-based splitmix64 generator shared with the device kernels.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3 = 0, 32, 64, 1088, 1120


def off_b3(npts: int = 4) -> int:
    return OFF_W3 + 32 * npts


def nparams(npts: int = 4) -> int:
    return off_b3(npts) + npts


NP, OFF_B3 = nparams(4), off_b3(4)  # the 4-point model
MODES = 32
N1 = 1024
PER_SAMPLE = 2 + 2 * MODES  # random draws per sample


def _splitmix64(z):
    z = (z + np.uint64(0x9E3779B97F4A7C15))
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, idx: np.ndarray) -> np.ndarray:
    """Same as the device generator: splitmix64(seed ^ idx*golden) -> [0,1)."""
    with np.errstate(over="ignore"):
        idx = np.asarray(idx, dtype=np.uint64)
        h = _splitmix64(np.uint64(seed) ^ (idx * np.uint64(0xD1B54A32D192ED03)))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def lagrange(npts: int, px: np.ndarray) -> np.ndarray:
    """Textbook Lagrange weights on nodes 0..npts-1 at px: shape (len(px), npts)."""
    px = np.asarray(px, dtype=np.float64)[:, None]
    out = np.ones((px.shape[0], npts))
    for j in range(npts):
        for m in range(npts):
            if m != j:
                out[:, j] *= (px[:, 0] - m) / (j - m)
    return out


def make_samples(n: int, seed: int, first: int = 0, n1: int = N1, npts: int = 4,
                 exact: bool = False):
    """(alpha, taps, target) of samples first .. first+n-1."""
    s = np.arange(first, first + n, dtype=np.uint64)
    base = s * np.uint64(PER_SAMPLE)
    x0 = uniform(seed, base)
    alpha = uniform(seed, base + np.uint64(1))
    k = np.arange(10, dtype=np.float64)
    x = x0[:, None] + (k[None, :] - 4.0) / n1
    xa = x0 + alpha / n1
    f = np.zeros((n, 10))
    fx = np.zeros(n)
    for m in range(1, MODES + 1):
        a = (2.0 * uniform(seed, base + np.uint64(2 * m)) - 1.0) / m
        b = (2.0 * uniform(seed, base + np.uint64(2 * m + 1)) - 1.0) / m
        ph = 2.0 * np.pi * m * x
        f += a[:, None] * np.cos(ph) + b[:, None] * np.sin(ph)
        fx += a * np.cos(2.0 * np.pi * m * xa) + b * np.sin(2.0 * np.pi * m * xa)
    target = fx if exact else (lagrange(10, 4.0 + alpha) * f).sum(1)
    k0 = 5 - npts // 2
    return alpha, f[:, k0:k0 + npts].copy(), target


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def unpack(p, npts: int = 4):
    p = np.asarray(p, dtype=np.float64)
    ob3 = off_b3(npts)
    return (p[OFF_W1:OFF_B1], p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(32, 32),
            p[OFF_B2:OFF_W3], p[OFF_W3:ob3].reshape(npts, 32), p[ob3:ob3 + npts])


def init_params(seed: int, npts: int = 4) -> np.ndarray:
    """Hidden layers: U[-1,1]*sqrt(6/(fan_in+fan_out)) from the shared
    generator; output layer zero (the model starts as Lagrange)."""
    n = nparams(npts)
    p = np.zeros(n)
    u = uniform(seed, np.arange(n, dtype=np.uint64))
    p[OFF_W1:OFF_B1] = (2 * u[OFF_W1:OFF_B1] - 1) * np.sqrt(6.0 / 33.0)
    p[OFF_W2:OFF_B2] = (2 * u[OFF_W2:OFF_B2] - 1) * np.sqrt(6.0 / 64.0)
    return p


def base_weights(npts: int, alpha) -> np.ndarray:
    """The Lagrange stencil the model corrects: nodes 0..npts-1 at npts/2 - 1 + a."""
    return lagrange(npts, (npts // 2 - 1) + np.asarray(alpha, dtype=np.float64))


def weights(p, alpha, npts: int = 4):
    W1, b1, W2, b2, W3, b3 = unpack(p, npts)
    a = np.asarray(alpha, dtype=np.float64)
    z1 = a[:, None] * W1[None, :] + b1[None, :]
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2[None, :]
    h2 = gelu(z2)
    c = h2 @ W3.T + b3[None, :]
    c = c - c.mean(1, keepdims=True)
    return base_weights(npts, a) + c


def loss_and_grad(p, alpha, taps, target):
    """Mean squared error and its gradient w.r.t. the parameters; the stencil
    size is taps.shape[1]."""
    npts = taps.shape[1]
    ob3 = off_b3(npts)
    W1, b1, W2, b2, W3, b3 = unpack(p, npts)
    a = np.asarray(alpha, dtype=np.float64)
    B = a.shape[0]
    z1 = a[:, None] * W1[None, :] + b1[None, :]
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2[None, :]
    h2 = gelu(z2)
    c = h2 @ W3.T + b3[None, :]
    w = base_weights(npts, a) + c - c.mean(1, keepdims=True)
    pred = (w * taps).sum(1)
    r = pred - target
    loss = float((r * r).mean())
    dpred = 2.0 * r / B
    dw = dpred[:, None] * taps
    dc = dw - dw.mean(1, keepdims=True)        # projection is symmetric
    g = np.zeros(nparams(npts))
    g[OFF_W3:ob3] = (dc.T @ h2).ravel()
    g[ob3:ob3 + npts] = dc.sum(0)
    dz2 = (dc @ W3) * gelu_grad(z2)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    g[OFF_W1:OFF_B1] = (dz1 * a[:, None]).sum(0)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g
