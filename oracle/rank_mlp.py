"""CPU restatement of the learned form's rank predictor (test infrastructure only).

The MLP 12 -> 64 -> 64 -> 1 with GELU (0.5 x (1 + erf(x / sqrt 2))), BF16 weights and the loss
L = (1/n) sum (y - t)^2, in float64 numpy with the weights rounded to BF16 (round to nearest even)
as the GPU kernels read them.  The backward pass is written out by hand (chain rule per layer),
independently of the CUDA code, so that the GPU gradients can be checked against it.  No
counterpart in the reference.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

F, H = 12, 64
SIZES = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("w3", (H,)), ("b3", (1,))]
P = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(params):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(params[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def bf16_round(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    r = ((b + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(params, X, rounded=True):
    w = unpack(bf16_round(params) if rounded else np.asarray(params, dtype=np.float64))
    a1 = X @ w["W1"].T + w["b1"]
    h1 = gelu(a1)
    a2 = h1 @ w["W2"].T + w["b2"]
    h2 = gelu(a2)
    return h2 @ w["w3"] + w["b3"][0], (a1, h1, a2, h2, w)


def gradient(params, X, T, rounded=True):
    """(dL/dparams, L) for L = (1/n) sum (y - t)^2, the derivative taken at the BF16 weights
    (rounded=True, as the GPU kernels) or at the parameters themselves."""
    X = np.asarray(X, dtype=np.float64)
    n = X.shape[0]
    y, (a1, h1, a2, h2, w) = forward(params, X, rounded)
    dy = 2.0 * (y - T) / n                       # dL/dy
    g = {"w3": h2.T @ dy, "b3": np.array([dy.sum()])}
    da2 = np.outer(dy, w["w3"]) * gelu_grad(a2)  # dL/da2
    g["W2"] = da2.T @ h1
    g["b2"] = da2.sum(axis=0)
    da1 = (da2 @ w["W2"]) * gelu_grad(a1)        # dL/da1
    g["W1"] = da1.T @ X
    g["b1"] = da1.sum(axis=0)
    flat = np.concatenate([g[name].ravel() for name, _ in SIZES])
    return flat, float(np.mean((y - T) ** 2))
