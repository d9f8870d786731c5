"""CPU oracle of the learned corrector's layers (test infrastructure only).

numpy restatement of every layer the corrector's CUDA kernels compute, forward and
backward, in float64 on BF16-rounded operands: the GPU kernels multiply BF16 values
exactly and accumulate in FP32, so the oracle isolates the accumulation error.  Only
tests/ and the bench's checks import this module.

Layouts as on the GPU: activations NHWC, weights [Cout][taps][Cin] with taps 9 (a 3 x 3
kernel, tap = 3 * (dy + 1) + (dx + 1)) or 1; "same" zero padding, stride 1.
"""
import numpy as np


def bf16_round(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_bits(a):
    """BF16 bit patterns (uint16) of float32 values, rounded to nearest even."""
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def _taps(taps):
    return [(0, 0)] if taps == 1 else [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _shift(x, dy, dx):
    """x[b, y + dy, x + dx, c] with zeros outside (NHWC)."""
    B, H, W, C = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[:, yd, xd, :] = x[:, ys, xs, :]
    return out


def conv2d(x, w, bias=None, relu=False):
    """y[b, y, x, co] = sum_{tap, ci} x[b, y + dy, x + dx, ci] w[co, tap, ci] (+ bias, ReLU)."""
    x = np.asarray(x, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    Cout, taps, Cin = w.shape
    y = np.zeros(x.shape[:3] + (Cout,))
    for t, (dy, dx) in enumerate(_taps(taps)):
        y += _shift(x, dy, dx) @ w[:, t, :].T
    if bias is not None:
        y += np.asarray(bias, dtype=np.float64)
    if relu:
        y = np.maximum(y, 0.0)
    return y


def conv2d_grad_input(gy, w):
    """dL/dx of conv2d for dL/dy = gy (no activation): sum over taps of gy shifted back."""
    gy = np.asarray(gy, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    Cout, taps, Cin = w.shape
    gx = np.zeros(gy.shape[:3] + (Cin,))
    for t, (dy, dx) in enumerate(_taps(taps)):
        gx += _shift(gy, -dy, -dx) @ w[:, t, :]
    return gx


def conv2d_grad_weight(x, gy, taps):
    """dL/dw[co, tap, ci] = sum_pixels gy[p, co] x[p + (dy, dx), ci]."""
    x = np.asarray(x, dtype=np.float64)
    gy = np.asarray(gy, dtype=np.float64)
    Cin, Cout = x.shape[3], gy.shape[3]
    gw = np.zeros((Cout, taps, Cin))
    g2 = gy.reshape(-1, Cout)
    for t, (dy, dx) in enumerate(_taps(taps)):
        gw[:, t, :] = g2.T @ _shift(x, dy, dx).reshape(-1, Cin)
    return gw


def conv2d_grad_bias(gy):
    return np.asarray(gy, dtype=np.float64).reshape(-1, gy.shape[-1]).sum(axis=0)


def avgpool2(x):
    B, H, W, C = x.shape
    x = np.asarray(x, dtype=np.float64)
    return 0.25 * ((x[:, 0::2, 0::2] + x[:, 0::2, 1::2]) + (x[:, 1::2, 0::2] + x[:, 1::2, 1::2]))


def avgpool2_bwd(gy):
    return 0.25 * np.repeat(np.repeat(np.asarray(gy, dtype=np.float64), 2, axis=1), 2, axis=2)


def upsample2(x):
    return np.repeat(np.repeat(np.asarray(x, dtype=np.float64), 2, axis=1), 2, axis=2)


def upsample2_bwd(gy):
    g = np.asarray(gy, dtype=np.float64)
    return (g[:, 0::2, 0::2] + g[:, 0::2, 1::2]) + (g[:, 1::2, 0::2] + g[:, 1::2, 1::2])
