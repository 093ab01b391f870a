"""CPU oracle of the learned endpoint proposal's network (TEST INFRASTRUCTURE ONLY).

The network has no counterpart in the reference; this is the FP64 statement of what the tensor-core
kernels compute, used by the tests to check the GPU forward pass and gradients. It follows the
library's arithmetic points: inputs, weights and every hidden activation (and, in the backward
pass, every activation gradient that feeds a matrix product) are rounded to BF16 where the kernels
round them; all sums are exact FP64 here.

Parameter layout (flat): W1 [256 x 48], b1 [256], W2 [256 x 256], b2 [256], W3 [8 x 256], b3 [8].
"""
import math

import numpy as np

IN, HID, OUT = 48, 256, 8
LOSS_WEIGHTS = np.array([1, 1, 1, 1, 1, 0.25, 0, 0], np.float64)


def bf16(x):
    """Round FP32 values to BF16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    nan = np.isnan(a)
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    parts = []
    for shape in [(HID, IN), (HID,), (HID, HID), (HID,), (OUT, HID), (OUT,)]:
        n = int(np.prod(shape))
        parts.append(p[o:o + n].reshape(shape))
        o += n
    return parts


# GELU in its tanh form (Hendrycks & Gimpel 2016), the network's activation, in float64.
GELU_S = math.sqrt(2.0 / math.pi)
GELU_C = 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GELU_S * (z + GELU_C * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GELU_S * (z + GELU_C * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_S * (1.0 + 3.0 * GELU_C * z * z)


def forward(p, x):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    xb = bf16(x)
    z1 = xb @ bf16(w1).T + b1
    h1 = bf16(gelu(z1))
    z2 = h1 @ bf16(w2).T + b2
    h2 = bf16(gelu(z2))
    y = h2 @ bf16(w3).T + b3
    return y, (xb, z1, h1, z2, h2)


def gradients(p, x, t):
    """Flat gradient of the weighted mean squared error and the loss."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    y, (xb, z1, h1, z2, h2) = forward(p, x)
    n = x.shape[0]
    w = LOSS_WEIGHTS / (n * OUT)
    d = y - np.asarray(t, np.float64)
    loss = float(np.sum(w * d * d))
    dy = 2.0 * w * d
    dyb = bf16(dy)
    dw3 = dyb.T @ h2
    db3 = dy.sum(axis=0)
    dz2 = (dyb @ bf16(w3)) * gelu_grad(z2)
    dz2b = bf16(dz2)
    dw2 = dz2b.T @ h1
    db2 = dz2.sum(axis=0)
    dz1 = (dz2b @ bf16(w2)) * gelu_grad(z1)
    dz1b = bf16(dz1)
    dw1 = dz1b.T @ xb
    db1 = dz1.sum(axis=0)
    return np.concatenate([dw1.ravel(), db1, dw2.ravel(), db2, dw3.ravel(), db3]), loss
