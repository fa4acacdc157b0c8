"""CPU oracle of the learned upscaler (test infrastructure).

numpy restatement of the network the CUDA kernels in
parallel-gs_gb300/csrc/upscaler.cu compute: 3x3 convolutions with zero padding,
activations and weights rounded to BF16 where the kernels store them, FP32/FP64
sums, mean-squared-error loss over the four channels, and the backward pass
(weight, bias and data gradients through the ReLUs).  Used only to check the
kernels' forward results and gradients.
"""
from __future__ import annotations

import numpy as np

SHAPES = [(4, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 4)]


def bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 to BF16 (nearest, ties to even), returned as FP32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray):
    layers, o = [], 0
    for cin, cout in SHAPES:
        w = params[o:o + 9 * cout * cin].reshape(9, cout, cin)
        o += 9 * cout * cin
        b = params[o:o + cout]
        o += cout
        layers.append((w, b))
    return layers


def shifted(x: np.ndarray, tap: int) -> np.ndarray:
    """x[n, y + dy - 1, x + dx - 1, :] with zeros outside."""
    dy, dx = tap // 3, tap % 3
    p = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    h, w = x.shape[1], x.shape[2]
    return p[:, dy:dy + h, dx:dx + w, :]


def conv(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    out = np.zeros(x.shape[:3] + (w.shape[1],), dtype=np.float64)
    for tap in range(9):
        out += shifted(x, tap).astype(np.float64) @ w[tap].T.astype(np.float64)
    return out


def conv_data_grad(dy: np.ndarray, w: np.ndarray) -> np.ndarray:
    """dX[q] = sum_tap dY[q - off(tap)] W[tap]^T (flipped taps)."""
    out = np.zeros(dy.shape[:3] + (w.shape[2],), dtype=np.float64)
    for tap in range(9):
        out += shifted(dy, 8 - tap).astype(np.float64) @ w[tap].astype(np.float64)
    return out


def weight_grad(x: np.ndarray, dy: np.ndarray) -> np.ndarray:
    """dW[tap][co][ci] = sum_p X[p + off(tap)][ci] dY[p][co]."""
    cin, cout = x.shape[3], dy.shape[3]
    g = np.zeros((9, cout, cin), dtype=np.float64)
    d = dy.reshape(-1, cout).astype(np.float64)
    for tap in range(9):
        g[tap] = d.T @ shifted(x, tap).reshape(-1, cin).astype(np.float64)
    return g


def forward(images: np.ndarray, params: np.ndarray):
    """images: (n, h, w, 4) uint8.  Returns (output, activations)."""
    layers = unpack(params)
    x0 = bf16(images.astype(np.float32) / np.float32(255.0))
    acts = [x0]
    a = x0
    for l, (w, b) in enumerate(layers[:-1]):
        z = conv(a, bf16(w)) + b
        a = bf16(np.maximum(z, 0.0))
        acts.append(a)
    w, b = layers[-1]
    out = conv(a, bf16(w)) + b + images.astype(np.float64) / 255.0
    return out, acts


def backward(images: np.ndarray, targets: np.ndarray, params: np.ndarray):
    """Returns (loss, flat gradient) of the mean squared error over all four channels."""
    layers = unpack(params)
    out, acts = forward(images, params)
    diff = out.astype(np.float64) - targets.astype(np.float64) / 255.0
    count = diff.size
    loss = float(np.sum(diff * diff) / count)
    g = bf16(2.0 * diff / count)
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        w, _ = layers[l]
        x = acts[l]
        grads[l] = (weight_grad(x, g), g.reshape(-1, g.shape[3]).astype(np.float64).sum(0))
        if l > 0:
            gx = conv_data_grad(g, bf16(w))
            g = bf16(np.where(acts[l] > 0, gx, 0.0))
    flat = np.concatenate([np.concatenate([gw.reshape(-1), gb]) for gw, gb in grads]).astype(np.float32)
    return loss, flat
