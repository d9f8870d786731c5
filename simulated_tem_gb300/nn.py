"""Python face of libstem_nn (include/stem_nn.h): the corrector's CUDA kernels on torch
device tensors.  torch provides device memory and streams only; every layer runs in the
library's own kernels, and a missing library is an error, never a fallback."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
NN_PATH = os.path.join(HERE, "libstem_nn.so")

_vp, _i32 = ctypes.c_void_p, ctypes.c_int32
_fp = ctypes.POINTER(ctypes.c_float)
_PROTOS = {
    "stn_conv2d_fwd": (_i32, [_vp, _i32, _i32, _i32, _i32, _vp, _i32, _i32, _vp, _i32, _vp, _i32, _vp]),
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


def conv2d(x, w, bias=None, relu=False, out_fp32=False, out=None):
    """NHWC BF16 x (B, H, W, Cin), weights (Cout, taps, Cin) BF16 -> (B, H, W, Cout)."""
    import torch
    B, H, W, Cin = x.shape
    Cout, taps, Cin_w = w.shape
    assert Cin_w == Cin and x.dtype == torch.bfloat16 and w.dtype == torch.bfloat16
    assert x.is_contiguous() and w.is_contiguous()
    if bias is not None:
        assert bias.dtype == torch.float32 and bias.is_contiguous() and bias.numel() == Cout
    if out is None:
        out = torch.empty((B, H, W, Cout), dtype=torch.float32 if out_fp32 else torch.bfloat16, device=x.device)
    _check(lib().stn_conv2d_fwd(_ptr(x), B, H, W, Cin, _ptr(w), Cout, taps, _ptr(bias), int(relu), _ptr(out),
                                int(out_fp32), _stream()), "stn_conv2d_fwd")
    return out


def last_kernel_error():
    return lib().stn_last_kernel_error()
