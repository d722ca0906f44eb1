"""CPU restatement of the MLP surrogate's forward / backward pass.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  Mirrors the GPU
pipeline's precision choices so gradients can be compared element-wise:
weights, inputs, activations and back-propagated gradients are rounded to
bfloat16 where the GPU stores them in bfloat16; products and sums are float64.

Network: x -> [Linear -> GELU] x H -> Linear, GELU(z) = z/2 (1 + erf(z/sqrt2)).
Loss: mean squared error over all outputs.
"""

import numpy as np
from scipy.special import erf


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def _ident(x):
    return np.asarray(x, dtype=np.float64)


def forward(Ws, bs, X, rounding=True):
    """Returns (Y, Zs, Hs): Hs[0] = bf16(X), Hs[l] = bf16(gelu(Z_l)).  With
    ``rounding=False`` everything stays float64 (exact-gradient checks)."""
    r = bf16 if rounding else _ident
    f32 = (lambda a: a.astype(np.float32).astype(np.float64)) if rounding else _ident
    H = r(X)
    Hs, Zs = [H], []
    L = len(Ws)
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Z = H @ r(W).T + b
        if l < L - 1:
            Zs.append(f32(Z))
            H = r(gelu(Z))
            Hs.append(H)
        else:
            Y = f32(Z)
    return Y, Zs, Hs


def backward(Ws, bs, X, T, rounding=True):
    """Gradients of mean((Y - T)^2) w.r.t. every W and b, and the loss."""
    r = bf16 if rounding else _ident
    f32 = (lambda a: a.astype(np.float32).astype(np.float64)) if rounding else _ident
    Y, Zs, Hs = forward(Ws, bs, X, rounding)
    n = Y.size
    dZ = 2.0 * (Y - T) / n
    loss = float(np.mean((Y - T) ** 2))
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for l in reversed(range(len(Ws))):
        dZb = r(dZ)
        gW[l] = dZb.T @ Hs[l]
        gb[l] = dZ.sum(axis=0)
        if l > 0:
            dH = dZb @ r(Ws[l])
            dZ = f32(dH * gelu_grad(Zs[l - 1]))
    return gW, gb, loss
