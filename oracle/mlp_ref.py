"""CPU reference of the surrogate network (TEST INFRASTRUCTURE ONLY).

float64 numpy forward/backward of the MLP 48 -> 128 -> 128 -> 16 (erf GELU) with the same
bfloat16 rounding points as the GPU training kernels: normalised inputs, hidden activations,
the output gradient and the pre-activation gradients are rounded to bf16 (round to nearest
even); weights are rounded to bf16 for the products; biases and accumulation stay wide.
Used to check the GPU gradients and the tensor-memory inference kernel.
"""
from __future__ import annotations

import math

import numpy as np

IN, H, OUT = 48, 128, 16
P_W1 = 0
P_B1 = P_W1 + H * IN
P_W2 = P_B1 + H
P_B2 = P_W2 + H * H
P_W3 = P_B2 + H
P_B3 = P_W3 + OUT * H
P_COUNT = P_B3 + OUT



def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even) and return them as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = rounded.astype(np.uint32).view(np.float32)
    out = np.where(np.isnan(a), a, out)
    return out.astype(np.float64)


K0 = math.sqrt(2.0 / math.pi)
K1 = 0.044715


def gelu(z):
    """GELU, tanh form (the device evaluates tanh with the hardware approximation)."""
    return 0.5 * z * (1.0 + np.tanh(K0 * (z + K1 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(K0 * (z + K1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * K0 * (1.0 + 3.0 * K1 * z * z)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[P_W1:P_B1].reshape(H, IN), p[P_B1:P_W2], p[P_W2:P_B2].reshape(H, H), p[P_B2:P_W3],
            p[P_W3:P_B3].reshape(OUT, H), p[P_B3:P_COUNT])


def normalise(x, y, norm):
    norm = np.asarray(norm, np.float32)
    mx, sx, my, sy = norm[:IN], norm[IN:2 * IN], norm[2 * IN:2 * IN + OUT], norm[2 * IN + OUT:]
    xn = bf16((np.asarray(x, np.float32) - mx) * sx)
    yn = ((np.asarray(y, np.float32) - my) * sy).astype(np.float64)
    return xn, yn


def grads(params, norm, x, y):
    """Gradients of mean((y_pred - y_norm)^2) over the batch and outputs, and the loss."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W1b, W2b, W3b = bf16(W1), bf16(W2), bf16(W3)
    xn, yn = normalise(x, y, norm)
    B = len(xn)
    z1 = xn @ W1b.T + b1
    h1 = bf16(gelu(z1))
    z2 = h1 @ W2b.T + b2
    h2 = bf16(gelu(z2))
    yp = h2 @ W3b.T + b3
    d = yp - yn
    loss = float(np.mean(d * d))
    dy32 = 2.0 * d / (B * OUT)
    dy = bf16(dy32)
    g = np.zeros(P_COUNT)
    g[P_W3:P_B3] = (dy.T @ h2).ravel()
    g[P_B3:P_COUNT] = dy32.sum(0)
    dh2 = dy @ W3b
    dz2_32 = dh2 * gelu_grad(z2)
    dz2 = bf16(dz2_32)
    g[P_W2:P_B2] = (dz2.T @ h1).ravel()
    g[P_B2:P_W3] = dz2_32.sum(0)
    dh1 = dz2 @ W2b
    dz1_32 = dh1 * gelu_grad(z1)
    dz1 = bf16(dz1_32)
    g[P_W1:P_B1] = (dz1.T @ xn).ravel()
    g[P_B1:P_W2] = dz1_32.sum(0)
    return g, loss


def infer(params, norm, x):
    """Increments predicted from raw features with the folded bf16 inference weights."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    norm = np.asarray(norm, np.float32)
    mx, sx, my, sy = norm[:IN], norm[IN:2 * IN], norm[2 * IN:2 * IN + OUT], norm[2 * IN + OUT:]
    W1f = bf16((W1 * sx).astype(np.float32))
    b1f = b1 - (W1 * sx) @ mx
    W3f = bf16((W3 / sy[:, None]).astype(np.float32))
    b3f = b3 / sy + my
    xb = bf16(x)
    h1 = bf16(gelu(xb @ W1f.T + b1f))
    h2 = bf16(gelu(h1 @ bf16(W2).T + b2))
    return h2 @ W3f.T + b3f
