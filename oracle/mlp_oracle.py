"""ORACLE — FP64 numpy restatement of the radiance-cache network.

Test infrastructure only (gradient and inference checks of the CUDA
kernels).  The reference's network lives in the un-vendored tiny-cuda-nn
submodule (no pinned revision is recorded in the reference tree), so this
restates the published algorithms the library implements: a fully
connected ReLU network without biases (the constant-1 input feature acts as
the first layer's bias), frequency encoding of the normalised position
(sin/cos of 2^j * pi * p, j = 0..11), exp output, the relative L2 loss of
Mueller et al., "Real-time Neural Radiance Caching for Path Tracing" (2021):
(p - y)^2 / (sg(p)^2 + 0.01), and Adam (Kingma & Ba, 2015).
Parity unpinned against the reference (no reference implementation here).
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT, LAYERS, FREQS = 96, 64, 16, 6, 12
DIMS = [(HID, IN)] + [(HID, HID)] * 4 + [(OUT, HID)]
PARAMS = sum(o * i for o, i in DIMS)


def split(params):
    out, off = [], 0
    for o, i in DIMS:
        out.append(np.asarray(params[off:off + o * i], np.float64).reshape(o, i))
        off += o * i
    return out


def join(ws):
    return np.concatenate([w.reshape(-1) for w in ws])


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(x, np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def encode(rec, lo, hi):
    rec = np.asarray(rec, np.float64)
    n = len(rec)
    inv = 1.0 / np.maximum(np.asarray(hi, np.float64) - np.asarray(lo, np.float64), 1e-6)
    p = (rec[:, 0:3] - np.asarray(lo, np.float64)) * inv
    x = np.zeros((n, IN))
    for a in range(3):
        for j in range(FREQS):
            v = np.pi * (2.0 ** j) * p[:, a]
            x[:, a * 24 + 2 * j] = np.sin(v)
            x[:, a * 24 + 2 * j + 1] = np.cos(v)
    x[:, 72:75] = rec[:, 4:7]
    x[:, 75:78] = rec[:, 8:11]
    x[:, 78] = rec[:, 3]
    x[:, 79:82] = rec[:, 12:15]
    x[:, 82] = 1.0
    return x


def forward(ws, x, emulate_bf16=False):
    """emulate_bf16: inputs and every hidden activation rounded to bfloat16,
    as the tensor-core kernels store them between layers."""
    r = bf16 if emulate_bf16 else (lambda v: v)
    a = r(x)
    acts, pre = [a], []
    for l in range(LAYERS - 1):
        z = a @ ws[l].T
        pre.append(z)
        a = r(np.maximum(z, 0.0))
        acts.append(a)
    z = a @ ws[-1].T
    return z, acts, pre


def predict(ws, x):
    z, _, _ = forward(ws, x)
    return np.exp(np.minimum(z[:, :3], 15.0))


def loss_and_grad(ws, x, y, den=None, emulate_bf16=False):
    """Relative L2 loss (mean over rows and RGB) and its weight gradient; the
    denominator sg(p)^2 + 0.01 is a constant of the gradient (stop-gradient),
    or the given `den`.  emulate_bf16 also rounds every dL/dz to bfloat16
    where the kernels store it."""
    r = bf16 if emulate_bf16 else (lambda v: v)
    n = len(x)
    z, acts, pre = forward(ws, x, emulate_bf16)
    p = np.exp(np.minimum(z[:, :3], 15.0))
    y = np.asarray(y, np.float64)[:, :3]
    if den is None:
        den = p * p + 0.01
    loss = np.sum((p - y) ** 2 / den) / (3 * n)
    dz = np.zeros_like(z)
    dz[:, :3] = 2.0 * (p - y) / den * p / (3 * n)
    grads = [None] * LAYERS
    d = r(dz)
    for l in range(LAYERS - 1, -1, -1):
        grads[l] = d.T @ acts[l]
        if l > 0:
            d = r((d @ ws[l]) * (pre[l - 1] > 0))
    return loss, grads
