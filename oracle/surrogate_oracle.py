"""CPU restatement of the surrogate network (test infrastructure only).

The reference has no learned surrogate; this module states the network that
the library's tensor-core kernels compute, so that their forward pass, loss
gradients and Adam step can be checked on the CPU.  Everything is FP64
except where the kernels round on purpose, which is emulated here exactly:

* operands of every matrix product are BF16 (round to nearest even): the
  Fourier features, the weights and the activations of the forward pass,
  and the activation gradients dH of the backward pass;
* pre-activations, biases, the output layer and the Adam masters are FP32
  values (computed here in FP64).

Parameter layout of one member (FP32, ``PARAM_COUNT`` values):
W1 [256][64], b1 [256], W2..W4 [256][256] each followed by its bias [256],
w5 [256], b5, zero padding to a multiple of 8.

Only the tests use this module, as the checker.
"""
from __future__ import annotations

import math

import numpy as np

N_IN = 7
N_FEAT = 64
WIDTH = 256
DEPTH = 4
IN_DIMS = (N_FEAT, WIDTH, WIDTH, WIDTH)
PARAM_COUNT = 214280


def offsets():
    """(weight offset, bias offset) of each hidden layer, then (w5, b5)."""
    out = []
    o = 0
    for k in IN_DIMS:
        out.append((o, o + WIDTH * k))
        o += WIDTH * k + WIDTH
    return out, (o, o + WIDTH)


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    from scipy.special import erf
    return 0.5 * x * (1.0 + erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    from scipy.special import erf
    return 0.5 * (1.0 + erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def unpack(p: np.ndarray):
    """Weights and biases of one member's parameter vector."""
    p = np.asarray(p, dtype=np.float64)
    hidden, (o5, ob5) = offsets()
    Ws, bs = [], []
    for (ow, ob), k in zip(hidden, IN_DIMS):
        Ws.append(p[ow:ow + WIDTH * k].reshape(WIDTH, k))
        bs.append(p[ob:ob + WIDTH])
    return Ws, bs, p[o5:o5 + WIDTH], p[ob5]


def features(x7: np.ndarray, B: np.ndarray) -> np.ndarray:
    """BF16 Fourier features [n][64]: sin then cos of 2 pi (B x), with B x
    accumulated in FP32 in input order as the feature kernel does."""
    x = np.asarray(x7, dtype=np.float32)
    Bf = np.asarray(B, dtype=np.float32)
    p = np.zeros((x.shape[0], Bf.shape[0]), dtype=np.float32)
    for q in range(N_IN):
        p = (p + Bf[None, :, q] * x[:, q:q + 1]).astype(np.float32)
    ang = 2.0 * math.pi * p.astype(np.float64)
    return np.concatenate([bf16(np.sin(ang)), bf16(np.cos(ang))], axis=1)


def forward(p: np.ndarray, X0: np.ndarray):
    """Pre-activations H_l, BF16 activations A_l and the output y of one member."""
    Ws, bs, w5, b5 = unpack(p)
    Hs, As = [], []
    a = X0
    for W, b in zip(Ws, bs):
        h = a @ bf16(W).T + b
        a = bf16(gelu(h))
        Hs.append(h)
        As.append(a)
    y = a @ w5 + b5
    return Hs, As, y


def loss_and_grads(p: np.ndarray, X0: np.ndarray, t: np.ndarray):
    """Mean squared error of one member on a batch and its parameter gradient,
    with the backward pass's BF16 rounding of dH."""
    Ws, bs, w5, b5 = unpack(p)
    Hs, As, y = forward(p, X0)
    n = X0.shape[0]
    diff = y - t
    loss = float(np.mean(diff * diff))
    g = 2.0 * diff / n
    grad = np.zeros(PARAM_COUNT)
    hidden, (o5, ob5) = offsets()
    grad[o5:o5 + WIDTH] = As[-1].T @ g
    grad[ob5] = g.sum()
    dH = bf16(g[:, None] * w5[None, :] * gelu_grad(Hs[-1]))
    for l in range(DEPTH - 1, -1, -1):
        a_in = X0 if l == 0 else As[l - 1]
        ow, ob = hidden[l]
        grad[ow:ow + WIDTH * IN_DIMS[l]] = (dH.T @ a_in).reshape(-1)
        grad[ob:ob + WIDTH] = dH.sum(axis=0)
        if l:
            dH = bf16((dH @ bf16(Ws[l])) * gelu_grad(Hs[l - 1]))
    return loss, y, grad


def adam_step(p, m, v, g, t: int, lr: float, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (step t counted from 1); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def cosine_lr(step: int, total: int, lr_max: float, lr_min: float) -> float:
    """Learning rate of 0-based step `step` under the library's cosine schedule."""
    frac = min(step / total, 1.0) if total else 0.0
    return lr_min + (lr_max - lr_min) * 0.5 * (1.0 + math.cos(math.pi * frac))
