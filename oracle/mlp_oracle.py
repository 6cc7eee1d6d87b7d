"""CPU oracle of the learned 4-point stencil (FP64 numpy). TEST INFRASTRUCTURE
ONLY: the checker for csrc/mlp.cu's data generator, forward, backward and
inference kernels.

Model (same layout as the CUDA kernels):
  params (1252 floats) = [W1 (32) | b1 (32) | W2 (32x32, [out][in]) | b2 (32) |
                          W3 (4x32, [out][in]) | b3 (4)]
  h1 = gelu(W1 * a + b1); h2 = gelu(W2 h1 + b2); c = W3 h2 + b3
  w(a) = lagrange3(a) + c - mean(c)        (the weights keep summing to 1)
  prediction = sum_k w_k * f[k], f = the 4 nodes j-1, j, j+1, j+2
  loss = mean over the batch of (prediction - target)^2
gelu(x) = x/2 (1 + erf(x/sqrt 2)).

Training samples: a random periodic line f(x) = sum_{m=1..M} a_m cos(2 pi m x)
+ b_m sin(2 pi m x), a_m, b_m ~ U[-1, 1]/m, 10 nodes x_k = x0 + (k-4)/n1
(k = 0..9), a shift a; the target is the degree-9 Lagrange interpolation of
the 10 nodes at 4 + a. Random numbers come from the counter-based splitmix64
generator shared with the device kernels.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

NP = 1252
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 32, 64, 1088, 1120, 1248
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


def make_samples(n: int, seed: int, first: int = 0):
    """(alpha, taps4, target) of samples first .. first+n-1."""
    s = np.arange(first, first + n, dtype=np.uint64)
    base = s * np.uint64(PER_SAMPLE)
    x0 = uniform(seed, base)
    alpha = uniform(seed, base + np.uint64(1))
    k = np.arange(10, dtype=np.float64)
    x = x0[:, None] + (k[None, :] - 4.0) / N1
    f = np.zeros((n, 10))
    for m in range(1, MODES + 1):
        a = (2.0 * uniform(seed, base + np.uint64(2 * m)) - 1.0) / m
        b = (2.0 * uniform(seed, base + np.uint64(2 * m + 1)) - 1.0) / m
        ph = 2.0 * np.pi * m * x
        f += a[:, None] * np.cos(ph) + b[:, None] * np.sin(ph)
    target = (lagrange(10, 4.0 + alpha) * f).sum(1)
    return alpha, f[:, 3:7].copy(), target


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1], p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(32, 32),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(4, 32), p[OFF_B3:NP])


def init_params(seed: int) -> np.ndarray:
    """Hidden layers: U[-1,1]*sqrt(6/(fan_in+fan_out)) from the shared
    generator; output layer zero (the model starts as Lagrange-3)."""
    p = np.zeros(NP)
    u = uniform(seed, np.arange(NP, dtype=np.uint64))
    p[OFF_W1:OFF_B1] = (2 * u[OFF_W1:OFF_B1] - 1) * np.sqrt(6.0 / 33.0)
    p[OFF_W2:OFF_B2] = (2 * u[OFF_W2:OFF_B2] - 1) * np.sqrt(6.0 / 64.0)
    return p


def weights(p, alpha):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    a = np.asarray(alpha, dtype=np.float64)
    z1 = a[:, None] * W1[None, :] + b1[None, :]
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2[None, :]
    h2 = gelu(z2)
    c = h2 @ W3.T + b3[None, :]
    c = c - c.mean(1, keepdims=True)
    return lagrange(4, 1.0 + a) + c


def loss_and_grad(p, alpha, taps4, target):
    """Mean squared error and its gradient w.r.t. the 1252 parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    a = np.asarray(alpha, dtype=np.float64)
    B = a.shape[0]
    z1 = a[:, None] * W1[None, :] + b1[None, :]
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2[None, :]
    h2 = gelu(z2)
    c = h2 @ W3.T + b3[None, :]
    w = lagrange(4, 1.0 + a) + c - c.mean(1, keepdims=True)
    pred = (w * taps4).sum(1)
    r = pred - target
    loss = float((r * r).mean())
    dpred = 2.0 * r / B
    dw = dpred[:, None] * taps4
    dc = dw - dw.mean(1, keepdims=True)        # projection is symmetric
    g = np.zeros(NP)
    g[OFF_W3:OFF_B3] = (dc.T @ h2).ravel()
    g[OFF_B3:NP] = dc.sum(0)
    dz2 = (dc @ W3) * gelu_grad(z2)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    g[OFF_W1:OFF_B1] = (dz1 * a[:, None]).sum(0)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g
