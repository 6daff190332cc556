"""ORACLE — test infrastructure only.

numpy restatement of the learned strategy picker's network (32 -> 64 -> 64 -> 3,
ReLU, bf16 weights with fp32 arithmetic, mean softmax cross-entropy), used to
check the CUDA forward and backward kernels.  Parameter layout (row-major,
out x in): W1, b1, W2, b2, W3, b3.
"""
from __future__ import annotations

import numpy as np

NF, H1, H2, NO = 32, 64, 64, 3
SIZES = [(H1, NF), (H1,), (H2, H1), (H2,), (NO, H2), (NO,)]
NPARAM = sum(int(np.prod(s)) for s in SIZES)


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest bfloat16 (ties to even), kept as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray):
    out, o = [], 0
    for s in SIZES:
        n = int(np.prod(s))
        out.append(p[o:o + n].reshape(s))
        o += n
    return out


def forward(p, X, bf16=True, dtype=np.float32):
    q = bf16_round(p) if bf16 else p
    W1, b1, W2, b2, W3, b3 = [a.astype(dtype) for a in unpack(q)]
    X = X.astype(dtype)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ W3.T + b3
    return z, (X, h1, h2, W2, W3)


def loss_and_grad(p, X, y, bf16=True, dtype=np.float32):
    z, (Xc, h1, h2, W2, W3) = forward(p, X, bf16, dtype)
    n = X.shape[0]
    zm = z - z.max(axis=1, keepdims=True)
    e = np.exp(zm)
    pr = e / e.sum(axis=1, keepdims=True)
    loss = float(-(zm[np.arange(n), y] - np.log(e.sum(axis=1))).mean())
    dz = pr.copy()
    dz[np.arange(n), y] -= 1
    dz /= n
    gW3 = dz.T @ h2
    gb3 = dz.sum(0)
    dh2 = (dz @ W3) * (h2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1 = dh1.T @ Xc
    gb1 = dh1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, g
