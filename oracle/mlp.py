"""CPU ORACLE for the moment-surrogate network -- TEST INFRASTRUCTURE ONLY.

A float64 numpy restatement of the network the GPU kernels in
cusna_gb300/csrc/mlp.cu train and evaluate (the reference has no surrogate, so
this restatement is the only oracle: "parity unpinned" against the reference,
pinned instead by central finite differences of its own loss):

  Z1 = X W1^T + b1,  H1 = gelu(Z1),  Z2 = H1 W2^T + b2,  H2 = gelu(Z2),
  Y  = H2 W3^T + b3,  loss = mean((Y - T)^2),  gelu(z) = z Phi(z).

With bf16=True every operand of a matrix product is rounded to bfloat16
(round to nearest even) first, as the tensor-core kernels round them, so the
GPU result differs from this one only by float32 accumulation. Parameters
are one flat vector laid out [W1 | b1 | W2 | b2 | W3 | b3].
"""
from __future__ import annotations

import math

import numpy as np

_SQRT1_2 = 1.0 / math.sqrt(2.0)
_INV_SQRT_2PI = 1.0 / math.sqrt(2.0 * math.pi)
_erf = np.vectorize(math.erf, otypes=[np.float64])


def bf16_round(a) -> np.ndarray:
    """Round float values to the nearest bfloat16 (ties to even), returned as
    float64. Operates on the float32 bit pattern: add 0x7FFF plus the lowest
    kept bit, then clear the 16 discarded bits."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z * _SQRT1_2))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z * _SQRT1_2)) + z * _INV_SQRT_2PI * np.exp(-0.5 * z * z)


def param_count(n_in, H, n_out):
    return H * n_in + H + H * H + H + n_out * H + n_out


def unpack(p, n_in, H, n_out):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = []
    for shape in ((H, n_in), (H,), (H, H), (H,), (n_out, H), (n_out,)):
        sz = int(np.prod(shape))
        out.append(p[o:o + sz].reshape(shape))
        o += sz
    return out


def forward(p, X, n_in, H, n_out, bf16=False):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, H, n_out)
    r = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    X = np.asarray(X, dtype=np.float64)
    Z1 = r(X) @ r(W1).T + b1
    H1 = gelu(Z1)
    Z2 = r(H1) @ r(W2).T + b2
    H2 = gelu(Z2)
    Y = r(H2) @ r(W3).T + b3
    return Y, (X, Z1, H1, Z2, H2)


def loss_grad(p, X, T, n_in, H, n_out, bf16=False):
    """(loss, gradient) of the mean squared error; the bf16 variant follows
    the kernels' rounding points (operands of each product, including the
    back-propagated errors)."""
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, H, n_out)
    r = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Y, (X, Z1, H1, Z2, H2) = forward(p, X, n_in, H, n_out, bf16)
    T = np.asarray(T, dtype=np.float64)
    B = X.shape[0]
    E = Y - T
    loss = float(np.mean(E * E))
    dY = 2.0 * E / (B * n_out)
    gW3 = r(dY).T @ r(H2)
    gb3 = dY.sum(axis=0)
    dZ2 = (r(dY) @ r(W3)) * gelu_grad(Z2)
    gW2 = r(dZ2).T @ r(H1)
    gb2 = dZ2.sum(axis=0)
    dZ1 = (r(dZ2) @ r(W2)) * gelu_grad(Z1)
    gW1 = r(dZ1).T @ r(X)
    gb1 = dZ1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def adam(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (Kingma & Ba 2015); returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def jacobian(p, X, n_in, H, n_out, n_wrt):
    """dY/dX[:, :n_wrt] per row, (B, n_out, n_wrt), exact float64 chain rule."""
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, H, n_out)
    _, (X, Z1, H1, Z2, H2) = forward(p, X, n_in, H, n_out)
    B = X.shape[0]
    J = np.zeros((B, n_out, n_wrt))
    for b in range(B):
        t1 = W1[:, :n_wrt] * gelu_grad(Z1[b])[:, None]
        t2 = (W2 @ t1) * gelu_grad(Z2[b])[:, None]
        J[b] = W3 @ t2
    return J
