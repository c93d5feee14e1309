"""CPU oracle of the learned closure's MLP (TEST INFRASTRUCTURE ONLY).

The closure has no counterpart in the reference, so this oracle restates our own definition
(particlesimulation_gb300/csrc/closure.cu): 67 inputs (padded to 80), three hidden layers of 64
with exact GELU, 3 outputs, parameters packed as W1 64x80, b1 64, W2 64x64, b2 64, W3 64x64,
b3 64, W4 8x64, b4 8.  Loss = mean over rows of |y - t|^2.

`forward` / `gradients` take `bf16=True` to round at the same points as the tensor-core kernels
(inputs, weights and activations to bfloat16, accumulation in wide precision; the output deltas
and hidden deltas to bfloat16 where the kernels feed them to the tensor cores); with
`bf16=False` they are the plain FP64 network, checked against finite differences by
tests/test_mlp_oracle.py.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

IN, K0, H, NO = 67, 80, 64, 8
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * K0
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + NO * H
NPARAM = OFF_B4 + NO


def bf16_round(a):
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, K0), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(H, H), p[OFF_B3:OFF_W4],
            p[OFF_W4:OFF_B4].reshape(NO, H), p[OFF_B4:NPARAM])


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


def _prep(p, x, bf16):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p)
    X = np.zeros((len(x), K0))
    X[:, :IN] = x
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    return r(X), r(W1), b1, r(W2), b2, r(W3), b3, r(W4), b4, r


def forward(p, x, bf16=True):
    X, W1, b1, W2, b2, W3, b3, W4, b4, r = _prep(p, x, bf16)
    z1 = X @ W1.T + b1
    a1 = r(gelu(z1))
    z2 = a1 @ W2.T + b2
    a2 = r(gelu(z2))
    z3 = a2 @ W3.T + b3
    a3 = r(gelu(z3))
    y = a3 @ W4.T + b4
    return y[:, :3], (X, z1, a1, z2, a2, z3, a3)


def loss(p, x, t, bf16=False):
    y, _ = forward(p, x, bf16)
    return float(((y - t) ** 2).sum(1).mean())


def gradients(p, x, t, bf16=True):
    X, W1, b1, W2, b2, W3, b3, W4, b4, r = _prep(p, x, bf16)
    y, (X, z1, a1, z2, a2, z3, a3) = forward(p, x, bf16)
    n = len(x)
    dy = np.zeros((n, NO))
    dy[:, :3] = 2.0 * (y - t) / n
    g = np.zeros(NPARAM)
    dyr = r(dy)
    g[OFF_W4:OFF_B4] = (dyr.T @ a3).reshape(-1)
    g[OFF_B4:NPARAM] = dy.sum(0)
    da = dyr @ W4
    for (z, a_in, off_w, off_b, W) in ((z3, a2, OFF_W3, OFF_B3, W3), (z2, a1, OFF_W2, OFF_B2, W2),
                                       (z1, X, OFF_W1, OFF_B1, None)):
        dz = da * gelu_grad(z)
        g[off_b:off_b + H] = dz.sum(0)
        dzr = r(dz)
        g[off_w:off_w + H * a_in.shape[1]] = (dzr.T @ a_in).reshape(-1)
        if W is not None:
            da = dzr @ W
    return g


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)

    def fill(off_w, rows, cols, rows_real, cols_real, off_b, fan_in):
        b = 1.0 / np.sqrt(fan_in)
        w = np.zeros((rows, cols), np.float32)
        w[:rows_real, :cols_real] = rng.uniform(-b, b, (rows_real, cols_real))
        p[off_w:off_w + rows * cols] = w.reshape(-1)
        p[off_b:off_b + rows_real] = rng.uniform(-b, b, rows_real)

    fill(OFF_W1, H, K0, H, IN, OFF_B1, IN)
    fill(OFF_W2, H, H, H, H, OFF_B2, H)
    fill(OFF_W3, H, H, H, H, OFF_B3, H)
    fill(OFF_W4, NO, H, 3, H, OFF_B4, H)
    return p
