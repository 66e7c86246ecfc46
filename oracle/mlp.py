"""Float64 CPU oracle of the proposal network's forward pass and loss gradient.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  The network has no
reference counterpart; this restates the mathematics the CUDA kernels in
``powerfit_gb300/csrc/pf_learn.cu`` implement, so that their forward values
and gradients can be checked:

    h1 = relu(W1 x + b1),  h2 = relu(W2 h1 + b2),  y = w3 . h2 + b3
    L  = sum_i c_i (y_i - t_i)^2,  c_i = scale * w_i

Parameters are the flat vector [W1 (H*F), b1 (H), W2 (H*H), b2 (H), w3 (H), b3].
"""
import numpy as np


def bf16_round(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(p, nin, nh):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + nh * nin].reshape(nh, nin); o += nh * nin
    b1 = p[o:o + nh]; o += nh
    W2 = p[o:o + nh * nh].reshape(nh, nh); o += nh * nh
    b2 = p[o:o + nh]; o += nh
    w3 = p[o:o + nh]; o += nh
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, x, nin, nh):
    W1, b1, W2, b2, w3, b3 = unpack(p, nin, nh)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    a2 = h1 @ W2.T + b2
    return np.maximum(a2, 0.0) @ w3 + b3


def loss_grad(p, x, t, w, scale, nin, nh):
    """(L, dL/dp) in float64."""
    W1, b1, W2, b2, w3, b3 = unpack(p, nin, nh)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    c = scale * (np.ones_like(t) if w is None else np.asarray(w, dtype=np.float64))
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ w3 + b3
    r = y - t
    L = float(np.sum(c * r * r))
    dy = 2.0 * c * r
    d2 = (dy[:, None] * w3[None, :]) * (a2 > 0)
    d1 = (d2 @ W2) * (h1 > 0)
    g = np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0),
                        h2.T @ dy, [dy.sum()]])
    return L, g
