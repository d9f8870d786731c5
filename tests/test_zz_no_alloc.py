"""st_blur_noalloc: the blur for callers that cannot let a library allocate GPU memory.

Such callers (a Fortran host whose MPI or batch runtime owns the device memory
pool, code with a fixed memory budget, code that must not allocate between
steps it replays) pass their own device buffers; the entry point keeps its
one intermediate in a fixed device array instead of allocating.  Its output
must equal st_blur's, bit for bit, on consecutive calls that reuse that array.
This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from simulated_tem_gb300 import _lib, imaging

pytestmark = pytest.mark.gpu


def _noalloc(L, img, t, stream):
    import torch
    nx, ny = img.shape
    d_in = torch.from_numpy(np.asfortranarray(img).ravel(order="F").copy()).cuda()
    d_out = torch.full_like(d_in, float("nan"))
    err = ctypes.create_string_buffer(256)
    torch.cuda.synchronize()
    rc = L.st_blur_noalloc(ctypes.c_void_p(d_in.data_ptr()), nx, ny, float(t), ctypes.c_void_p(d_out.data_ptr()),
                           ctypes.c_void_p(stream), err, 256)
    torch.cuda.synchronize()
    return rc, err.value.decode(), d_out.cpu().numpy().reshape((nx, ny), order="F")


def test_blur_noalloc_matches_st_blur_on_consecutive_calls():
    import torch
    L = _lib.lib()
    ctx = imaging.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2024)
    try:
        # a large image, then a smaller one that reuses the array the first call left behind;
        # then the limits: the widest weight table (t near 204.6 px, an 8 KB kernel argument)
        # and the widest and largest image the scratch takes (nx = 4096, nx * ny = 2^21)
        for nx, ny, t in ((566, 566, 3.1446), (94, 131, 2.5), (300, 220, 204.0),
                          (_lib.ST_BLUR_NOALLOC_MAX_NX, _lib.ST_BLUR_NOALLOC_MAX_PIXELS // _lib.ST_BLUR_NOALLOC_MAX_NX,
                           4.7)):
            img = rng.random((nx, ny))
            want = ctx.blur(img, t)
            rc, msg, got = _noalloc(L, img, t, stream)
            assert rc == _lib.ST_OK, msg
            assert np.array_equal(got, want)
    finally:
        ctx.close()


def test_blur_noalloc_rejects_images_beyond_its_scratch():
    import torch
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    nx, ny = 2048, _lib.ST_BLUR_NOALLOC_MAX_PIXELS // 2048 + 1
    d = torch.zeros(1, dtype=torch.float64, device="cuda")  # never read: the size check comes first
    err = ctypes.create_string_buffer(256)
    rc = L.st_blur_noalloc(ctypes.c_void_p(d.data_ptr()), nx, ny, 2.0, ctypes.c_void_p(d.data_ptr()),
                           ctypes.c_void_p(stream), err, 256)
    assert rc == _lib.ST_ERR_ARG
    assert b"exceeds the fixed scratch" in err.value
