"""CPU oracle of the control-variate MLP (test infrastructure).

The network has no reference counterpart (the reference computes every local
energy exactly); this numpy restatement is the checker of the GPU's forward and
backward kernels: x (67) -> SiLU(W1 x + b1) (256) -> SiLU(W2 h1 + b2) (256) ->
w3 . h2 + b3, mean-squared-error loss.  Weights of the forward pass are
rounded to BF16, as on the GPU; arithmetic is FP64 here.
"""
import numpy as np


def bf16_round(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x):
    W1, b1, W2, b2, w3, b3 = params
    z1 = x @ bf16_round(W1).astype(np.float64).T + b1
    h1 = silu(z1)
    z2 = h1 @ bf16_round(W2).astype(np.float64).T + b2
    h2 = silu(z2)
    y = h2 @ bf16_round(w3).astype(np.float64) + b3[0]
    return y, (z1, h1, z2, h2)


def loss_and_grads(params, x, t):
    """MSE loss (1/B) sum (y - t)^2 and its gradients w.r.t. all parameters."""
    W1, b1, W2, b2, w3, b3 = params
    x = np.asarray(x, np.float64)
    B = x.shape[0]
    y, (z1, h1, z2, h2) = forward(params, x)
    r = y - t
    loss = float((r * r).mean())
    dy = 2.0 * r / B
    gw3 = h2.T @ dy
    gb3 = np.array([dy.sum()])
    dh2 = np.outer(dy, bf16_round(w3).astype(np.float64))
    dz2 = dh2 * dsilu(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dh1 = dz2 @ bf16_round(W2).astype(np.float64)
    dz1 = dh1 * dsilu(z1)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    return loss, [gW1, gb1, gW2, gb2, gw3, gb3]
