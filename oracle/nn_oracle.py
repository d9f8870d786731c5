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


# ---------------------------------------------------------------------------
# The corrector network (simulated_tem_gb300/corrector.py)
# ---------------------------------------------------------------------------
# In float64 throughout, or (bf16=True) with every tensor the GPU stores in BF16 rounded
# to BF16 at the same point: convolution outputs after bias and ReLU, pooled and summed
# tensors, the loss gradient and every gradient passed between layers.

def _rounder(bf16):
    if not bf16:
        return lambda a: a
    return lambda a: bf16_round(np.asarray(a, dtype=np.float32)).astype(np.float64)


def unet_forward(P, x, ch=(32, 64, 128, 256), bf16=False):
    """Activations of the U-Net for input x (B, H, W, 16); P maps "<layer>.w" (Cout, taps,
    Cin) and "<layer>.b" (Cout,) to arrays."""
    r = _rounder(bf16)

    def conv(name, x, relu):
        y = conv2d(x, P[name + ".w"], P[name + ".b"])
        return r(np.maximum(y, 0.0)) if relu else y

    a = {"x0": np.asarray(x, dtype=np.float64)}
    a["e0a"] = conv("enc0a", a["x0"], True)
    a["e0"] = conv("enc0b", a["e0a"], True)
    a["p1"] = r(avgpool2(a["e0"]))
    a["e1a"] = conv("enc1a", a["p1"], True)
    a["e1"] = conv("enc1b", a["e1a"], True)
    a["p2"] = r(avgpool2(a["e1"]))
    a["e2a"] = conv("enc2a", a["p2"], True)
    a["e2"] = conv("enc2b", a["e2a"], True)
    a["p3"] = r(avgpool2(a["e2"]))
    a["e3a"] = conv("bota", a["p3"], True)
    a["e3"] = conv("botb", a["e3a"], True)
    a["c2"] = np.concatenate([upsample2(a["e3"]), a["e2"]], axis=3)
    a["d2a"] = conv("dec2a", a["c2"], True)
    a["d2"] = conv("dec2b", a["d2a"], True)
    a["c1"] = np.concatenate([upsample2(a["d2"]), a["e1"]], axis=3)
    a["d1a"] = conv("dec1a", a["c1"], True)
    a["d1"] = conv("dec1b", a["d1a"], True)
    a["c0"] = np.concatenate([upsample2(a["d1"]), a["e0"]], axis=3)
    a["d0a"] = conv("dec0a", a["c0"], True)
    a["d0"] = conv("dec0b", a["d0a"], True)
    a["out"] = conv("head", a["d0"], False)
    return a


def unet_loss_grads(P, x, target, ch=(32, 64, 128, 256), bf16=False):
    """MSE loss mean_p (out[p, 0] - target[p])^2 and its gradients for every parameter."""
    r = _rounder(bf16)
    a = unet_forward(P, x, ch, bf16)
    d = a["out"][..., 0] - target
    loss = float((d ** 2).mean())
    g_out = np.zeros_like(a["out"])
    g_out[..., 0] = 2.0 * d / d.size
    g_out = r(g_out)
    G = {}

    def layer(name, x_in, g_pre, mask=None, need_dx=True):
        taps = P[name + ".w"].shape[1]
        G[name + ".w"] = conv2d_grad_weight(x_in, g_pre, taps)
        G[name + ".b"] = conv2d_grad_bias(g_pre)
        if not need_dx:
            return None
        gx = conv2d_grad_input(g_pre, P[name + ".w"])
        return r(gx * (mask > 0) if mask is not None else gx)

    c0, c1, c2, c3 = ch
    g = layer("head", a["d0"], g_out, a["d0"])
    g = layer("dec0b", a["d0a"], g, a["d0a"])
    g = layer("dec0a", a["c0"], g, a["c0"])
    g_d1, g_e0 = r(upsample2_bwd(g[..., :c1])), g[..., c1:]
    g = layer("dec1b", a["d1a"], g_d1, a["d1a"])
    g = layer("dec1a", a["c1"], g, a["c1"])
    g_d2, g_e1 = r(upsample2_bwd(g[..., :c2])), g[..., c2:]
    g = layer("dec2b", a["d2a"], g_d2, a["d2a"])
    g = layer("dec2a", a["c2"], g, a["c2"])
    g_e3, g_e2 = r(upsample2_bwd(g[..., :c3])), g[..., c3:]
    g = layer("botb", a["e3a"], g_e3, a["e3a"])
    g = layer("bota", a["p3"], g)
    g = r(r(avgpool2_bwd(g)) + g_e2) * (a["e2"] > 0)
    g = layer("enc2b", a["e2a"], g, a["e2a"])
    g = layer("enc2a", a["p2"], g)
    g = r(r(avgpool2_bwd(g)) + g_e1) * (a["e1"] > 0)
    g = layer("enc1b", a["e1a"], g, a["e1a"])
    g = layer("enc1a", a["p1"], g)
    g = r(r(avgpool2_bwd(g)) + g_e0) * (a["e0"] > 0)
    g = layer("enc0b", a["e0a"], g, a["e0a"])
    layer("enc0a", a["x0"], g, need_dx=False)
    return loss, G
