"""CPU restatement of the redistribution surrogate's arithmetic (test
infrastructure: only tests/, the smoke check and bench.py's checks import it).

The network is 4 -> 128 -> 128 -> 32 with ReLU and a softmax.  Each input row
(s, u, r, cap) -- s = sigma_theta / dtheta in [0, 8], u in [0, 1), r =
sigma_E / centre spacing in [0, 4], cap 0 or 1 -- is scaled to [-1, 1] and
fed as 16 values: the bf16 rounding of each scaled feature, 128 x its
rounding remainder (also rounded to bf16), then zeros.  The weights of the
remainder columns 4-7 are tied to columns 0-3: bf16(W1[:, i]) / 128 (their
own parameters stay zero), so the first layer forms bf16(W1[:, i]) times the
input to about 16 bits.  The GPU kernels hold
every GEMM operand in bf16 (inputs, weights, hidden activations, loss
gradients) and accumulate in fp32; this module rounds the same operands to
bf16 (round to nearest even) and does the rest in float64, so the two differ
by the order of fp32 accumulation only.  Loss: mean softmax cross-entropy
against soft targets.
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 16, 128, 32
O_W1 = 0
O_W2 = O_W1 + HID * IN
O_W3 = O_W2 + HID * HID
O_B1 = O_W3 + OUT * HID
O_B2 = O_B1 + HID
O_B3 = O_B2 + HID
N_PARAMS = O_B3 + OUT
S_MAX, R_MAX = 8.0, 4.0


def scaled(feats):
    """[n][4] feature rows -> the scaled inputs in [-1, 1] (float64)."""
    f = np.asarray(feats, np.float64).reshape(-1, 4)
    return np.stack([2.0 * np.clip(f[:, 0], 0.0, S_MAX) / S_MAX - 1.0, 2.0 * f[:, 1] - 1.0,
                     2.0 * np.clip(f[:, 2], 0.0, R_MAX) / R_MAX - 1.0, 2.0 * f[:, 3] - 1.0], axis=1)


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(params):
    p = np.asarray(params, np.float32)
    return (p[O_W1:O_W2].reshape(HID, IN), p[O_W2:O_W3].reshape(HID, HID), p[O_W3:O_B1].reshape(OUT, HID),
            p[O_B1:O_B2], p[O_B2:O_B3], p[O_B3:N_PARAMS])


def w1_image(W1):
    """The first layer's bf16 weights as the GPU image holds them: columns 4-7
    are bf16(W1[:, 0:4]) / 128 (exact, a power of two)."""
    w = bf16(W1).copy()
    w[:, 4:8] = w[:, 0:4] / np.float32(128.0)
    return w


def tie_w1_grad(g):
    """Gradient of the tied parameterisation: d/dW1[:, i] gains 1/128 of the
    remainder column's gradient; columns 4-7 have none."""
    g = np.array(g, np.float64, copy=True)
    w = g[O_W1:O_W2].reshape(HID, IN)
    w[:, 0:4] += w[:, 4:8] / 128.0
    w[:, 4:8] = 0.0
    return g


def features(feats):
    """[n][4] physical inputs -> [n][16] network inputs (bf16 hi/lo pairs)."""
    f = np.asarray(feats, np.float32).reshape(-1, 4)
    s = np.minimum(np.maximum(f[:, 0], np.float32(0.0)), np.float32(S_MAX))
    r = np.minimum(np.maximum(f[:, 2], np.float32(0.0)), np.float32(R_MAX))
    u = np.stack([np.float32(2.0) * s / np.float32(S_MAX) - np.float32(1.0), np.float32(2.0) * f[:, 1] - np.float32(1.0),
                  np.float32(2.0) * r / np.float32(R_MAX) - np.float32(1.0),
                  np.float32(2.0) * f[:, 3] - np.float32(1.0)], axis=1).astype(np.float32)
    hi = bf16(u)
    lo = bf16((u - hi) * np.float32(128.0))
    x = np.zeros((f.shape[0], IN), np.float32)
    x[:, :4] = hi
    x[:, 4:8] = lo
    return x


def forward(params, feats):
    """Softmax tables [n][32] and the intermediates of the backward pass."""
    W1, W2, W3, b1, b2, b3 = unpack(params)
    x = features(feats).astype(np.float64)
    h1 = bf16(np.maximum(x @ w1_image(W1).T.astype(np.float64) + b1, 0.0).astype(np.float32)).astype(np.float64)
    h2 = bf16(np.maximum(h1 @ bf16(W2).T.astype(np.float64) + b2, 0.0).astype(np.float32)).astype(np.float64)
    z = h2 @ bf16(W3).T.astype(np.float64) + b3
    z = z - z.max(axis=1, keepdims=True)
    e = np.exp(z)
    p = e / e.sum(axis=1, keepdims=True)
    return p, (x, h1, h2, z)


FLOOR = 1.0 / 4096.0   # inference: weights below 2^-12 are zero


def table(params, feats):
    """The inference kernel's tables [n][32]: the softmax with weights below
    FLOOR set to zero and the largest weight taking 1 - the others (each row
    sums to 1)."""
    p, _ = forward(params, feats)
    p = np.where(p < FLOOR, 0.0, p)
    am = p.argmax(axis=1)
    rows = np.arange(p.shape[0])
    p[rows, am] = 0.0
    p[rows, am] = 1.0 - p.sum(axis=1)
    return p


def loss_and_grad(params, feats, target):
    """Mean cross-entropy and its gradient in the fp32 parameter layout."""
    W1, W2, W3, b1, b2, b3 = unpack(params)
    y = np.asarray(target, np.float64)
    n = y.shape[0]
    p, (x, h1, h2, z) = forward(params, feats)
    logp = z - np.log(np.exp(z).sum(axis=1, keepdims=True))
    loss = -(y * logp).sum() / n
    d3 = bf16(((p - y) / n).astype(np.float32)).astype(np.float64)
    g = np.zeros(N_PARAMS, np.float64)
    g[O_W3:O_B1] = (d3.T @ h2).ravel()
    g[O_B3:] = d3.sum(axis=0)
    dh2 = d3 @ bf16(W3).astype(np.float64)
    d2 = bf16(np.where(h2 > 0, dh2, 0.0).astype(np.float32)).astype(np.float64)
    g[O_W2:O_W3] = (d2.T @ h1).ravel()
    g[O_B2:O_B3] = d2.sum(axis=0)
    dh1 = d2 @ bf16(W2).astype(np.float64)
    d1 = bf16(np.where(h1 > 0, dh1, 0.0).astype(np.float32)).astype(np.float64)
    g[O_W1:O_W2] = (d1.T @ x).ravel()
    g[O_B1:O_B2] = d1.sum(axis=0)
    return loss, tie_w1_grad(g)


def loss_exact(params, feats, target):
    """The same loss without any bf16 rounding (float64 throughout), for finite differences."""
    W1, W2, W3, b1, b2, b3 = [np.asarray(a, np.float64) for a in unpack(params)]
    f = np.asarray(feats, np.float64).reshape(-1, 4)
    x = np.zeros((f.shape[0], IN))
    x[:, :4] = scaled(f)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    z = h2 @ W3.T + b3
    z = z - z.max(axis=1, keepdims=True)
    logp = z - np.log(np.exp(z).sum(axis=1, keepdims=True))
    return -(np.asarray(target, np.float64) * logp).sum() / f.shape[0]


def grad_exact(params, feats, target):
    """Analytic float64 gradient of loss_exact (lo inputs zero)."""
    W1, W2, W3, b1, b2, b3 = [np.asarray(a, np.float64) for a in unpack(params)]
    f = np.asarray(feats, np.float64).reshape(-1, 4)
    y = np.asarray(target, np.float64)
    n = f.shape[0]
    x = np.zeros((n, IN))
    x[:, :4] = scaled(f)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    z = h2 @ W3.T + b3
    z = z - z.max(axis=1, keepdims=True)
    p = np.exp(z) / np.exp(z).sum(axis=1, keepdims=True)
    d3 = (p - y) / n
    g = np.zeros(N_PARAMS)
    g[O_W3:O_B1] = (d3.T @ h2).ravel()
    g[O_B3:] = d3.sum(axis=0)
    d2 = np.where(h2 > 0, d3 @ W3, 0.0)
    g[O_W2:O_W3] = (d2.T @ h1).ravel()
    g[O_B2:O_B3] = d2.sum(axis=0)
    d1 = np.where(h1 > 0, d2 @ W2, 0.0)
    g[O_W1:O_W2] = (d1.T @ x).ravel()
    g[O_B1:O_B2] = d1.sum(axis=0)
    return g


def adam(params, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step in float32, as the update kernel does it."""
    p = np.asarray(params, np.float32).copy()
    g = np.asarray(grad, np.float32)
    m = (np.float32(b1) * m + np.float32(1 - b1) * g).astype(np.float32)
    v = (np.float32(b2) * v + np.float32(1 - b2) * g * g).astype(np.float32)
    bc1 = np.float32(1 - b1 ** t)
    bc2 = np.float32(1 - b2 ** t)
    p -= np.float32(lr) * (m / bc1) / (np.sqrt(v / bc2) + np.float32(eps))
    return p, m, v


def init_params(seed=12345):
    """The library's initial weights: He-uniform from its LCG, zero biases."""
    p = np.zeros(N_PARAMS, np.float32)
    st = seed

    def u():
        nonlocal st
        st = (1664525 * st + 1013904223) & 0xFFFFFFFF
        return np.float32((np.float32(st >> 8) + np.float32(0.5)) * np.float32(1.0 / 16777216.0))

    for k in range(O_W1, O_W2):
        p[k] = (np.float32(2.0) * u() - np.float32(1.0)) * np.float32(np.sqrt(np.float32(6.0 / 8.0)))
    p[O_W1:O_W2].reshape(HID, IN)[:, 4:8] = 0.0   # tied to columns 0-3
    for k in range(O_W2, O_W3):
        p[k] = (np.float32(2.0) * u() - np.float32(1.0)) * np.float32(np.sqrt(np.float32(6.0 / HID)))
    for k in range(O_W3, O_B1):
        p[k] = (np.float32(2.0) * u() - np.float32(1.0)) * np.float32(np.sqrt(np.float32(1.0 / HID)))
    return p
