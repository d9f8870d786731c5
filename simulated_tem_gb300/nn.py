"""Python face of libstem_nn (include/stem_nn.h): the corrector's CUDA kernels on torch
device tensors.  torch provides device memory and streams only; every layer runs in the
library's own kernels, and a missing library is an error, never a fallback."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
NN_PATH = os.path.join(HERE, "libstem_nn.so")

_vp, _i32 = ctypes.c_void_p, ctypes.c_int32
_fp = ctypes.POINTER(ctypes.c_float)
_i64, _f32 = ctypes.c_int64, ctypes.c_float
_PROTOS = {
    "stn_conv2d_fwd": (_i32, [_vp, _i32, _i32, _i32, _i32, _vp, _i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp]),
    "stn_conv2d_wgrad_workspace": (_i64, [_i32, _i32, _i32, _i32, _i32, _i32]),
    "stn_conv2d_wgrad": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _i64, _vp]),
    "stn_bias_grad_workspace": (_i64, [_i32]),
    "stn_weight_flip": (_i32, [_vp, _vp, _i32, _i32, _i32, _vp]),
    "stn_avgpool2": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "stn_avgpool2_bwd": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "stn_upsample2": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "stn_upsample2_bwd": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "stn_concat": (_i32, [_vp, _vp, _vp, _i64, _i32, _i32, _vp]),
    "stn_upsample2_concat": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "stn_split": (_i32, [_vp, _vp, _vp, _i64, _i32, _i32, _vp]),
    "stn_relu_mask": (_i32, [_vp, _vp, _i64, _vp]),
    "stn_bias_grad": (_i32, [_vp, _vp, _i64, _i32, _vp, _i64, _vp]),
    "stn_mse": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _i32, _f32, _vp]),
    "stn_adam": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _f32, _f32, _f32, _f32, _i32, _f32, _vp]),
    "stn_pack": (_i32, [_vp, _i32, _vp, _i64, _i32, _vp]),
    "stn_to_bf16": (_i32, [_vp, _vp, _i64, _vp]),
    "stn_add": (_i32, [_vp, _vp, _i64, _vp]),
    "stn_fill_zero": (_i32, [_vp, _i64, _vp]),
    "stn_image_mean": (_i32, [_vp, _i64, _vp, _vp]),
    "stn_resample_planes": (_i32, [_vp, _i32, _i32, _i32, _i32, _i32, _i32, _f32, _vp, _f32, _vp, _vp]),
    "stn_apply_correction": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _f32, _vp, _vp]),
    "stn_tile_maxabs": (_i32, [_vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _vp]),
    "stn_tile_flags": (_i32, [_vp, _i32, _i32, _f32, _i32, _vp, _vp, _vp]),
    "stn_merge_tiles": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp]),
    "stn_last_kernel_error": (_i32, []),
}
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(NN_PATH):
            raise RuntimeError("libstem_nn.so is not built (run simulated_tem_gb300/build.py)")
        L = ctypes.CDLL(NN_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


class NNError(RuntimeError):
    pass


def _check(code, what):
    if code != 0:
        raise NNError("%s failed (code %d)" % (what, code))


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else t.data_ptr()


def _bf16_empty(shape, like):
    import torch
    return torch.empty(shape, dtype=torch.bfloat16, device=like.device)


def conv2d(x, w, bias=None, relu=False, out_fp32=False, out=None, mask=None):
    """NHWC BF16 x (B, H, W, Cin), weights (Cout, taps, Cin) BF16 -> (B, H, W, Cout)."""
    import torch
    B, H, W, Cin = x.shape
    Cout, taps, Cin_w = w.shape
    assert Cin_w == Cin and x.dtype == torch.bfloat16 and w.dtype == torch.bfloat16
    assert x.is_contiguous() and w.is_contiguous()
    if bias is not None:
        assert bias.dtype == torch.float32 and bias.is_contiguous() and bias.numel() == Cout
    if mask is not None:
        assert mask.shape == (B, H, W, Cout) and mask.dtype == torch.bfloat16 and mask.is_contiguous()
    if out is None:
        out = torch.empty((B, H, W, Cout), dtype=torch.float32 if out_fp32 else torch.bfloat16, device=x.device)
    _check(lib().stn_conv2d_fwd(_ptr(x), B, H, W, Cin, _ptr(w), Cout, taps, _ptr(bias), int(relu), _ptr(mask),
                                _ptr(out), int(out_fp32), _stream()), "stn_conv2d_fwd")
    return out


_WORKSPACE = {}


def _workspace(floats, device):
    """An FP32 device buffer of at least `floats` values, kept per device (grown, never
    shrunk); callers use it on one stream at a time."""
    import torch
    key = str(device)
    buf = _WORKSPACE.get(key)
    if buf is None or buf.numel() < floats:
        buf = torch.empty(max(int(floats), 1), dtype=torch.float32, device=device)
        _WORKSPACE[key] = buf
    return buf


def conv2d_wgrad(x, gy, taps, gw):
    """gw (Cout, taps, Cin) FP32 += weight gradient of a convolution with input x, output gradient gy."""
    B, H, W, Cin = x.shape
    Cout = gy.shape[3]
    assert gy.shape[:3] == x.shape[:3] and gw.shape == (Cout, taps, Cin)
    n = lib().stn_conv2d_wgrad_workspace(B, H, W, Cin, Cout, taps)
    if n <= 0:
        raise NNError("stn_conv2d_wgrad_workspace: invalid arguments")
    ws = _workspace(n, x.device)
    _check(lib().stn_conv2d_wgrad(_ptr(x), _ptr(gy), B, H, W, Cin, Cout, taps, _ptr(gw), _ptr(ws), ws.numel(),
                                  _stream()), "stn_conv2d_wgrad")
    return gw


def weight_flip(w, out=None):
    """(Cout, taps, Cin) -> (Cin, taps, Cout) with the taps reversed."""
    Cout, taps, Cin = w.shape
    if out is None:
        out = _bf16_empty((Cin, taps, Cout), w)
    _check(lib().stn_weight_flip(_ptr(w), _ptr(out), Cout, taps, Cin, _stream()), "stn_weight_flip")
    return out


def conv2d_dgrad(gy, wt, mask=None, out=None):
    """Input gradient of a convolution: conv of gy with flipped weights wt, masked by mask > 0."""
    return conv2d(gy, wt, out=out, mask=mask)


def avgpool2(x, out=None):
    B, H, W, C = x.shape
    out = _bf16_empty((B, H // 2, W // 2, C), x) if out is None else out
    _check(lib().stn_avgpool2(_ptr(x), _ptr(out), B, H, W, C, _stream()), "stn_avgpool2")
    return out


def avgpool2_bwd(gy, out=None):
    B, H2, W2, C = gy.shape
    out = _bf16_empty((B, 2 * H2, 2 * W2, C), gy) if out is None else out
    _check(lib().stn_avgpool2_bwd(_ptr(gy), _ptr(out), B, 2 * H2, 2 * W2, C, _stream()), "stn_avgpool2_bwd")
    return out


def upsample2(x, out=None):
    B, H, W, C = x.shape
    out = _bf16_empty((B, 2 * H, 2 * W, C), x) if out is None else out
    _check(lib().stn_upsample2(_ptr(x), _ptr(out), B, H, W, C, _stream()), "stn_upsample2")
    return out


def upsample2_bwd(gy, out=None):
    B, H2, W2, C = gy.shape
    out = _bf16_empty((B, H2 // 2, W2 // 2, C), gy) if out is None else out
    _check(lib().stn_upsample2_bwd(_ptr(gy), _ptr(out), B, H2 // 2, W2 // 2, C, _stream()), "stn_upsample2_bwd")
    return out


def concat(a, b, out=None):
    B, H, W, Ca = a.shape
    Cb = b.shape[3]
    out = _bf16_empty((B, H, W, Ca + Cb), a) if out is None else out
    _check(lib().stn_concat(_ptr(a), _ptr(b), _ptr(out), B * H * W, Ca, Cb, _stream()), "stn_concat")
    return out


def upsample2_concat(d, e, out=None):
    """concat(upsample2(d), e) in one pass (d at half the resolution of e)."""
    B, H, W, Ce = e.shape
    Cd = d.shape[3]
    assert d.shape[:3] == (B, H // 2, W // 2)
    out = _bf16_empty((B, H, W, Cd + Ce), e) if out is None else out
    _check(lib().stn_upsample2_concat(_ptr(d), _ptr(e), _ptr(out), B, H, W, Cd, Ce, _stream()),
           "stn_upsample2_concat")
    return out


def split(gy, Ca, ga=None, gb=None):
    B, H, W, C = gy.shape
    _check(lib().stn_split(_ptr(gy), _ptr(ga), _ptr(gb), B * H * W, Ca, C - Ca, _stream()), "stn_split")
    return ga, gb


def relu_mask(g, y):
    _check(lib().stn_relu_mask(_ptr(g), _ptr(y), g.numel(), _stream()), "stn_relu_mask")
    return g


def bias_grad(g, gb):
    C = g.shape[-1]
    ws = _workspace(lib().stn_bias_grad_workspace(C), g.device)
    _check(lib().stn_bias_grad(_ptr(g), _ptr(gb), g.numel() // C, C, _ptr(ws), ws.numel(), _stream()),
           "stn_bias_grad")
    return gb


def mse(pred, target, g, loss, w1=0.0, target1=None):
    """loss (FP32 scalar tensor) += mean (pred[..., 0] - target)^2 + w1 mean (pred[..., 1] -
    t1)^2 with t1 = target1 or |target|; g = its gradient (BF16)."""
    Cp = pred.shape[-1]
    _check(lib().stn_mse(_ptr(pred), _ptr(target), _ptr(target1), _ptr(g), _ptr(loss), pred.numel() // Cp, Cp,
                         float(w1), _stream()), "stn_mse")
    return loss


def adam(w, m, v, g, step, lr, w16=None, beta1=0.9, beta2=0.999, eps=1e-8, wd=0.0):
    _check(lib().stn_adam(_ptr(w), _ptr(m), _ptr(v), _ptr(g), _ptr(w16), w.numel(), lr, beta1, beta2, eps, step, wd,
                          _stream()), "stn_adam")


def pack(planes, C, out=None):
    """FP32 planes (n, B, H, W) -> NHWC BF16 (B, H, W, C)."""
    n = planes.shape[0]
    B, H, W = planes.shape[1:]
    out = _bf16_empty((B, H, W, C), planes) if out is None else out
    _check(lib().stn_pack(_ptr(planes), n, _ptr(out), B * H * W, C, _stream()), "stn_pack")
    return out


def to_bf16(x, out=None):
    import torch
    out = torch.empty(x.shape, dtype=torch.bfloat16, device=x.device) if out is None else out
    _check(lib().stn_to_bf16(_ptr(x), _ptr(out), x.numel(), _stream()), "stn_to_bf16")
    return out


def last_kernel_error():
    return lib().stn_last_kernel_error()


def add_(a, b):
    """a += b (BF16)."""
    _check(lib().stn_add(_ptr(a), _ptr(b), a.numel(), _stream()), "stn_add")
    return a


def zero_(t):
    _check(lib().stn_fill_zero(_ptr(t), t.numel() * t.element_size(), _stream()), "stn_fill_zero")
    return t


def image_mean(img, out):
    _check(lib().stn_image_mean(_ptr(img), img.numel(), _ptr(out), _stream()), "stn_image_mean")
    return out


def resample_planes(img2, Mx2, My2, Mx8, My8, Wp, Hp, sg_value, mean, contrast, planes):
    """img2: FP64 device image (Mx2 x My2 column-major); mean: FP64 device scalar; planes:
    FP32 (5, Hp, Wp)."""
    _check(lib().stn_resample_planes(_ptr(img2), Mx2, My2, Mx8, My8, Wp, Hp, float(sg_value), _ptr(mean),
                                     float(contrast), _ptr(planes), _stream()), "stn_resample_planes")
    return planes


def apply_correction(base, pred, Mx8, My8, scale, out):
    Hp, Wp = base.shape[-2:]
    _check(lib().stn_apply_correction(_ptr(base), _ptr(pred), pred.shape[-1], Mx8, My8, Wp, float(scale), _ptr(out),
                                      _stream()), "stn_apply_correction")
    return out


def tile_maxabs(pred, Mx8, My8, T, out, ch=0):
    Wp = pred.shape[-2]
    _check(lib().stn_tile_maxabs(_ptr(pred), pred.shape[-1], ch, Mx8, My8, Wp, T, _ptr(out), _stream()),
           "stn_tile_maxabs")
    return out


def tile_flags(tile_max, thresh, mask, count, border=True):
    """mask (uint8, tile_max's shape) = tile_max > thresh (compared in FP32), or the tile on
    the outer ring; count (int32 device scalar) = the flagged tiles.  No host round trip."""
    nty, ntx = tile_max.shape
    _check(lib().stn_tile_flags(_ptr(tile_max), ntx, nty, float(thresh), int(bool(border)), _ptr(mask), _ptr(count),
                                _stream()), "stn_tile_flags")
    return mask


def merge_tiles(fine, mask, T, Mx, My, out):
    _check(lib().stn_merge_tiles(_ptr(fine), _ptr(mask), mask.shape[-1], T, Mx, My, _ptr(out), _stream()),
           "stn_merge_tiles")
    return out
