"""CPU restatement of the learned scheduler's network arithmetic (numpy).

Test infrastructure only: the GPU kernels of pdfs_gb300/csrc/mlp.cu are
checked against these functions.  The scheduler has no counterpart in the
reference (it sweeps every node), so this oracle restates the library's own
definition of the network: 16 -> 64 (ReLU) -> 64 (ReLU) -> 1, bf16 weights
and activations (round to nearest even), sums accumulated in wider precision
(float64 here, FP32 on the GPU), mean weighted binary cross-entropy, Adam
with bias correction.  With round=False every bf16 rounding is skipped, so
the backward pass can be checked against finite differences in float64.
"""
from __future__ import annotations

import numpy as np

NI, NH = 16, 64
NP = NH * NI + NH + NH * NH + NH + NH + 1


def bf16(a):
    """float32 values rounded to bf16 precision (round to nearest even)."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def bf16_bits(a):
    """bf16 bit patterns (uint16) of float32 values (round to nearest even)."""
    return (bf16(a).view(np.uint32) >> 16).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32)


def unpack(p):
    """Flat parameters -> (W1[64,16], b1, W2[64,64], b2, w3, b3)."""
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + NH * NI].reshape(NH, NI); o += NH * NI
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    w3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])


def _r(a, round_):
    return bf16(a).astype(np.float64) if round_ else np.asarray(a, dtype=np.float64)


def forward(p, x, round_=True):
    """Logits z and the activations (h1, h2) of samples x[n, 16]."""
    W1, b1, W2, b2, w3, b3 = unpack(_r(p, round_))
    x = _r(x, round_)
    h1 = _r(np.maximum(x @ W1.T + b1, 0.0), round_)
    h2 = _r(np.maximum(h1 @ W2.T + b2, 0.0), round_)
    return h2 @ w3 + b3, h1, h2


def loss_grad(p, x, y, pos_weight, round_=True):
    """Mean weighted cross-entropy and its gradient (flat, float64)."""
    W1, b1, W2, b2, w3, b3 = unpack(_r(p, round_))
    xr = _r(x, round_)
    z, h1, h2 = forward(p, x, round_)
    n = len(z)
    y = np.asarray(y, dtype=np.float64)
    wy = np.where(y > 0, pos_weight, 1.0)
    loss = float(np.sum(wy * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))) / n)
    pz = 1.0 / (1.0 + np.exp(-z))
    dz = wy * (pz - y) / n
    dh2 = (h2 > 0) * dz[:, None] * w3[None, :]
    dh1 = _r((h1 > 0) * (dh2 @ W2), round_)
    g = pack(dh1.T @ xr, dh1.sum(0), dh2.T @ h1, dh2.sum(0), (dz[:, None] * h2).sum(0), dz.sum())
    return loss, g


def adam(p, m, v, g, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step in float32 throughout, as the GPU computes it: the
    decay rates are float32, 1 - b is formed in float32, and the bias
    corrections are 1 - b**step in float32.  Returns (p, m, v)."""
    p, m, v, g = (np.asarray(a, dtype=np.float32) for a in (p, m, v, g))
    one, b1, b2 = np.float32(1), np.float32(b1), np.float32(b2)
    m = b1 * m + (one - b1) * g
    v = b2 * v + (one - b2) * g * g
    bc1 = one - b1 ** np.float32(step)
    bc2 = one - b2 ** np.float32(step)
    p = p - np.float32(lr) * (m / bc1) / (np.sqrt(v / bc2) + np.float32(eps))
    return p, m, v
