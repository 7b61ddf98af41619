"""ORACLE (test infrastructure only): FP64 numpy statement of the learned T2
initialiser's network, for checking the GPU forward and backward kernels.

Same parameter layout and arithmetic as the device code: features normalised
with (mu, sd); W1 and W2 are used rounded to BF16 (the device keeps BF16
working copies of them), w3 and the biases in FP32; GELU(x) = x Phi(x) with
the exact normal CDF; loss = mean squared error.  With ``bf16_ops=True`` the
other operand of every tensor-core product is rounded to BF16 as well (the
device stages both operands of its mma.sync products in BF16): the
normalised features and H1 in the forward pass, dZ2, H1, dZ1 and the
features in the gradient products.  The output layer (w3) and the bias
gradients stay unrounded, as on the device.
"""
from __future__ import annotations

import math

import numpy as np

NF, H = 16, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * NF
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
OFF_MU = OFF_B3 + 1
OFF_SD = OFF_MU + NF
NPARAM = OFF_SD + NF
NTRAIN = OFF_MU


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP64."""
    f = np.asarray(x, dtype=np.float32).copy()
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def _phi(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu(x):
    return x * _phi(x)


def gelu_grad(x):
    return _phi(x) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def unpack(p: np.ndarray):
    p = np.asarray(p, dtype=np.float64)
    W1 = bf16_round(p[OFF_W1:OFF_B1].astype(np.float32)).reshape(H, NF)
    b1 = p[OFF_B1:OFF_W2]
    W2 = bf16_round(p[OFF_W2:OFF_B2].astype(np.float32)).reshape(H, H)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    mu = p[OFF_MU:OFF_SD]
    sd = p[OFF_SD:NPARAM]
    return W1, b1, W2, b2, w3, b3, mu, sd


def _op(x, bf16_ops):
    """A tensor-core operand: rounded to BF16 when the device does so."""
    return bf16_round(np.asarray(x, dtype=np.float32)) if bf16_ops else x


def forward(p, Xraw, bf16_ops: bool = False):
    W1, b1, W2, b2, w3, b3, mu, sd = unpack(p)
    X = (np.asarray(Xraw, dtype=np.float64) - mu) / sd
    Z1 = _op(X, bf16_ops) @ W1.T + b1
    H1 = gelu(Z1)
    Z2 = _op(H1, bf16_ops) @ W2.T + b2
    H2 = gelu(Z2)
    y = H2 @ w3 + b3
    return y, (X, Z1, H1, Z2, H2)


def loss_and_grad(p, Xraw, target, bf16_ops: bool = False):
    W1, b1, W2, b2, w3, b3, mu, sd = unpack(p)
    y, (X, Z1, H1, Z2, H2) = forward(p, Xraw, bf16_ops)
    B = len(target)
    d = y - np.asarray(target, dtype=np.float64)
    loss = float(np.mean(d * d))
    dy = 2.0 * d / B
    g = np.zeros(NTRAIN)
    g[OFF_W3:OFF_B3] = H2.T @ dy
    g[OFF_B3] = dy.sum()
    dZ2 = np.outer(dy, w3) * gelu_grad(Z2)
    g[OFF_W2:OFF_B2] = (_op(dZ2, bf16_ops).T @ _op(H1, bf16_ops)).ravel()
    g[OFF_B2:OFF_W3] = dZ2.sum(axis=0)
    dZ1 = (_op(dZ2, bf16_ops) @ W2) * gelu_grad(Z1)
    g[OFF_W1:OFF_B1] = (_op(dZ1, bf16_ops).T @ _op(X, bf16_ops)).ravel()
    g[OFF_B1:OFF_W2] = dZ1.sum(axis=0)
    return loss, g
