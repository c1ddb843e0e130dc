"""CPU restatement of the calibration-step network (test infrastructure only:
the checker of the tcgen05 kernels in watergap2_gb300/csrc/wg_mlp.cu).

Same arithmetic as the GPU: inputs, weights and hidden activations rounded to
BF16 (round to nearest even), products accumulated in wide precision, biases
and the output in FP32; ReLU masks taken from the rounded activations; weight
gradients from BF16 dZ and activations, bias gradients from the unrounded dZ.
Parameter layout as include/wg_mlp.h.
"""
from __future__ import annotations

import numpy as np

W = 128
OUT = 16
LAYER_OUT = (W, W, W, OUT)


def bf16(a) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(theta):
    out, o = [], 0
    for n_out in LAYER_OUT:
        w = theta[o:o + n_out * W].reshape(n_out, W)
        o += n_out * W
        b = theta[o:o + n_out]
        o += n_out
        out.append((w, b))
    return out


def num_params() -> int:
    return sum(n * W + n for n in LAYER_OUT)


def forward(theta, x):
    """Returns y [n][16] and the BF16 hidden activations."""
    layers = unpack(np.asarray(theta, np.float32))
    a = bf16(x).astype(np.float64)
    hs = []
    for l, (w, b) in enumerate(layers):
        z = a @ bf16(w).astype(np.float64).T + b.astype(np.float64)
        if l < 3:
            a = bf16(np.maximum(z, 0.0).astype(np.float32)).astype(np.float64)
            hs.append(a)
        else:
            y = z.astype(np.float32)
    return y, hs


def gradient(theta, x, target):
    """Gradient of sum((y[:, :k] - target)^2) / n (k = target columns) and the loss."""
    theta = np.asarray(theta, np.float32)
    layers = unpack(theta)
    n, k = target.shape
    y, hs = forward(theta, x)
    e = y[:, :k].astype(np.float64) - target
    loss = float((e * e).sum() / n)
    g = np.zeros((n, OUT))
    g[:, :k] = 2.0 * e / n
    xb = bf16(x).astype(np.float64)
    grads = [None] * 4
    for l in range(3, -1, -1):
        w, _ = layers[l]
        dz = g if l == 3 else g * (hs[l] > 0)
        db = dz.sum(axis=0)
        dzb = bf16(dz.astype(np.float32)).astype(np.float64)
        a_in = hs[l - 1] if l > 0 else xb
        dw = dzb.T @ a_in
        grads[l] = (dw, db)
        if l > 0:
            g = dzb @ bf16(w).astype(np.float64)
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return flat.astype(np.float32), loss
