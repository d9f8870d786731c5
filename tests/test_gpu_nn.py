"""The corrector's tensor-core kernels against the CPU oracle (oracle/nn_oracle.py).

Operands are BF16 (exact products), accumulation FP32: with FP32 output the bar is
1e-5 of the output's magnitude (FP32 summation of up to 2,304 products); with BF16
output, one BF16 rounding (2^-8 relative) on top.
"""
import numpy as np
import pytest

from oracle import nn_oracle as NO

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _bf16(a):
    return torch.from_numpy(NO.bf16_round(a)).to(torch.bfloat16).cuda()


def _rand(rng, *shape, scale=1.0):
    return NO.bf16_round(rng.standard_normal(shape).astype(np.float32) * scale)


@pytest.fixture(scope="module")
def nn():
    from simulated_tem_gb300 import nn as N
    N.lib()
    return N


@pytest.mark.parametrize("B,H,W,Cin,Cout,taps", [
    (1, 1, 256, 64, 64, 1),     # a GEMM: 256 x 64 x 64
    (2, 1, 200, 128, 256, 1),   # ragged M, two N tiles of 128
    (1, 16, 16, 32, 64, 9),
    (2, 13, 17, 16, 32, 9),     # ragged image, KC = 16
    (1, 24, 20, 64, 128, 9),
    (1, 12, 12, 128, 16, 9),    # Cout 16 in a 32-wide tile
    (1, 13, 20, 192, 64, 9),    # two-row tiles (BN 64), odd height: the last tile's second row is outside
    (2, 7, 9, 160, 40, 9),      # two-row tiles, Cout 40 in a 64-wide tile
    (1, 5, 33, 256, 24, 1),     # two-row tiles of a 1 x 1 convolution
])
def test_conv_fwd_matches_oracle(nn, B, H, W, Cin, Cout, taps):
    rng = np.random.default_rng(B * 1000 + Cin + Cout + taps)
    x = _rand(rng, B, H, W, Cin)
    w = _rand(rng, Cout, taps, Cin, scale=1.0 / np.sqrt(taps * Cin))
    bias = rng.standard_normal(Cout).astype(np.float32)
    want = NO.conv2d(x, w, bias)
    got = nn.conv2d(_bf16(x), _bf16(w), torch.from_numpy(bias).cuda(), relu=False, out_fp32=True)
    torch.cuda.synchronize()
    assert nn.last_kernel_error() == 0
    got = got.cpu().numpy().astype(np.float64)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 1e-5 * scale
    # BF16 output with ReLU: one rounding of the FP32 result
    got16 = nn.conv2d(_bf16(x), _bf16(w), torch.from_numpy(bias).cuda(), relu=True).float().cpu().numpy()
    ref = np.maximum(want, 0.0)
    assert np.all(np.abs(got16 - ref) <= np.abs(ref) * 2.0 ** -8 + 1e-5 * scale)


@pytest.mark.parametrize("B,H,W,Cin,Cout,taps", [
    (1, 16, 16, 32, 64, 9),
    (2, 13, 17, 16, 32, 9),
    (1, 20, 24, 64, 128, 9),
    (1, 12, 12, 128, 256, 9),
    (2, 1, 300, 64, 32, 1),
])
def test_conv_backward_matches_oracle(nn, B, H, W, Cin, Cout, taps):
    """Input gradient (flipped weights + masked forward convolution) and weight gradient."""
    rng = np.random.default_rng(7 * B + H + Cin + Cout)
    x = NO.bf16_round(np.maximum(rng.standard_normal((B, H, W, Cin)).astype(np.float32), 0.0))  # post-ReLU
    w = _rand(rng, Cout, taps, Cin, scale=1.0 / np.sqrt(taps * Cin))
    gy = _rand(rng, B, H, W, Cout)
    # input gradient, masked by the ReLU that produced x
    wt = nn.weight_flip(_bf16(w))
    got = nn.conv2d(_bf16(gy), wt, mask=_bf16(x), out_fp32=True).cpu().numpy()
    want = NO.conv2d_grad_input(gy, w) * (x > 0)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
    # weight gradient (FP32, accumulated into zeros)
    gw = torch.zeros((Cout, taps, Cin), dtype=torch.float32, device="cuda")
    nn.conv2d_wgrad(_bf16(x), _bf16(gy), taps, gw)
    torch.cuda.synchronize()
    assert nn.last_kernel_error() == 0
    want_w = NO.conv2d_grad_weight(x, gy, taps)
    assert np.abs(gw.cpu().numpy() - want_w).max() <= 1e-5 * np.abs(want_w).max() + 1e-6
    # the partial sums of the pixel split are added in a fixed order: the same bits every time
    gw2 = torch.zeros_like(gw)
    nn.conv2d_wgrad(_bf16(x), _bf16(gy), taps, gw2)
    assert torch.equal(gw, gw2)


def test_elementwise_layers_match_oracle(nn):
    rng = np.random.default_rng(11)
    x = _rand(rng, 2, 8, 12, 32)
    g = _rand(rng, 2, 4, 6, 32)
    assert np.allclose(nn.avgpool2(_bf16(x)).float().cpu().numpy(), NO.bf16_round(NO.avgpool2(x).astype(np.float32)))
    assert np.allclose(nn.avgpool2_bwd(_bf16(g)).float().cpu().numpy(),
                       NO.bf16_round(NO.avgpool2_bwd(g).astype(np.float32)))
    assert np.array_equal(nn.upsample2(_bf16(g)).float().cpu().numpy(), NO.upsample2(g))
    assert np.allclose(nn.upsample2_bwd(_bf16(x)).float().cpu().numpy(),
                       NO.bf16_round(NO.upsample2_bwd(x).astype(np.float32)))
    # the decoder's fused input: concat(upsample2(d), e)
    d, e = _rand(rng, 2, 4, 6, 32), _rand(rng, 2, 8, 12, 16)
    assert np.array_equal(nn.upsample2_concat(_bf16(d), _bf16(e)).float().cpu().numpy(),
                          np.concatenate([NO.upsample2(d), e], axis=3))
    a, b = _rand(rng, 2, 5, 7, 16), _rand(rng, 2, 5, 7, 24)
    cat = nn.concat(_bf16(a), _bf16(b))
    assert np.array_equal(cat.float().cpu().numpy(), np.concatenate([a, b], axis=3))
    ga = torch.empty((2, 5, 7, 16), dtype=torch.bfloat16, device="cuda")
    gb = torch.empty((2, 5, 7, 24), dtype=torch.bfloat16, device="cuda")
    nn.split(cat, 16, ga, gb)
    assert np.array_equal(ga.float().cpu().numpy(), a) and np.array_equal(gb.float().cpu().numpy(), b)
    gm = _bf16(x)
    nn.relu_mask(gm, _bf16(np.abs(x) - 0.5))
    assert np.array_equal(gm.float().cpu().numpy(), x * (np.abs(x) - 0.5 > 0))
    gbias = torch.zeros(32, dtype=torch.float32, device="cuda")
    nn.bias_grad(_bf16(x), gbias)
    assert np.allclose(gbias.cpu().numpy(), NO.conv2d_grad_bias(x), rtol=1e-5, atol=1e-4)
    gbias2 = torch.zeros_like(gbias)
    nn.bias_grad(_bf16(x), gbias2)
    assert torch.equal(gbias, gbias2)
    # wide layers: more channels than threads of a block
    big = _rand(rng, 3, 7, 9, 512)
    gbig = torch.zeros(512, dtype=torch.float32, device="cuda")
    nn.bias_grad(_bf16(big), gbig)
    assert np.allclose(gbig.cpu().numpy(), NO.conv2d_grad_bias(big), rtol=1e-5, atol=1e-4)
    pred = rng.standard_normal((3, 9, 10, 16)).astype(np.float32)
    tgt = rng.standard_normal((3, 9, 10)).astype(np.float32)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    gl = torch.empty((3, 9, 10, 16), dtype=torch.bfloat16, device="cuda")
    nn.mse(torch.from_numpy(pred).cuda(), torch.from_numpy(tgt).cuda(), gl, loss, w1=0.5)
    d = pred[..., 0].astype(np.float64) - tgt
    d1 = pred[..., 1].astype(np.float64) - np.abs(tgt)
    want = (d ** 2).mean() + 0.5 * (d1 ** 2).mean()
    assert abs(loss.item() - want) <= 1e-5 * want
    glh = gl.float().cpu().numpy()
    assert np.allclose(glh[..., 0], NO.bf16_round((2 * d / d.size).astype(np.float32)), rtol=0, atol=1e-7)
    assert np.allclose(glh[..., 1], NO.bf16_round((0.5 * 2 * d1 / d1.size).astype(np.float32)), rtol=0, atol=1e-7)
    assert not glh[..., 2:].any()


@pytest.mark.parametrize("nty,ntx,border", [(142, 142, True), (1, 1, True), (3, 37, False), (40, 1, True)])
def test_tile_flags_and_merge(nn, nty, ntx, border):
    """The fallback mask made on the device: above the threshold (FP32 compare, ties not
    flagged) or on the outer ring; its count; the merge of the fine tiles it selects."""
    rng = np.random.default_rng(nty * 1000 + ntx)
    tm = rng.random((nty, ntx)).astype(np.float32)
    thresh = 0.7
    tm.flat[::7] = np.float32(thresh)  # ties with the threshold
    want = tm > np.float32(thresh)
    if border:
        want[0, :] = want[-1, :] = want[:, 0] = want[:, -1] = True
    mask = torch.empty((nty, ntx), dtype=torch.uint8, device="cuda")
    count = torch.empty((), dtype=torch.int32, device="cuda")
    nn.tile_flags(torch.from_numpy(tm).cuda(), thresh, mask, count, border=border)
    assert np.array_equal(mask.cpu().numpy(), want.astype(np.uint8))
    assert count.item() == int(want.sum())
    T = 8
    Mx, My = ntx * T - 3, nty * T - 5 if nty * T > 5 else nty * T  # ragged last tiles
    fine = torch.from_numpy(rng.random((My, Mx))).cuda()
    out = torch.from_numpy(rng.random((My, Mx))).cuda()
    exp = out.cpu().numpy().copy()
    sel = np.repeat(np.repeat(want, T, 0), T, 1)[:My, :Mx]
    exp[sel] = fine.cpu().numpy()[sel]
    nn.merge_tiles(fine, mask, T, Mx, My, out)
    assert np.array_equal(out.cpu().numpy(), exp)


def test_conv_streams_take_turns_on_blocked_weights(nn):
    """Layers of the halo-tile kernel copy their weights into one library buffer first:
    convolutions of different weights queued on two streams without synchronising give
    the results of the same calls made one at a time (bit for bit)."""
    rng = np.random.default_rng(21)
    x = _bf16(_rand(rng, 1, 24, 40, 192))
    ws = [_bf16(_rand(rng, 128, 9, 192, scale=0.02)), _bf16(_rand(rng, 64, 9, 192, scale=0.02))]
    want = [nn.conv2d(x, w, out_fp32=True) for w in ws]
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    outs = []
    for i in range(8):
        with torch.cuda.stream(streams[i % 2]):
            outs.append(nn.conv2d(x, ws[i % 2], out_fp32=True))
    torch.cuda.synchronize()
    assert nn.last_kernel_error() == 0
    for i, o in enumerate(outs):
        assert torch.equal(o, want[i % 2])


def test_input_planes_mean_and_pack(nn):
    """The corrector's input path against numpy: the coarse image's mean (one fixed-order
    FP64 sum), the planes resampled bilinearly onto the fine grid in FP64 (past the last
    coarse pixel the last two extrapolate, the padding rows and columns repeat the last
    pixel), and their BF16 NHWC packing
    (exact: one rounding of each FP32 value, zeros past the planes)."""
    rng = np.random.default_rng(5)
    Mx2, My2, Mx8, My8, Wp, Hp = 37, 29, 147, 115, 152, 120
    img2 = 0.1 + 0.6 * rng.random((My2, Mx2))  # numpy (My2, Mx2) = column-major (Mx2, My2)
    d_img2 = torch.from_numpy(img2).cuda()
    mean = torch.empty(1, dtype=torch.float64, device="cuda")
    nn.image_mean(d_img2, mean)
    mu = img2.mean()
    assert abs(mean.item() - mu) <= 1e-14 * mu
    planes = torch.empty((5, Hp, Wp), dtype=torch.float32, device="cuda")
    nn.resample_planes(d_img2, Mx2, My2, Mx8, My8, Wp, Hp, 0.25, mean, 20.0, planes)
    px = np.minimum(np.arange(Wp), Mx8 - 1)
    py = np.minimum(np.arange(Hp), My8 - 1)
    u, v = px * (Mx2 / Mx8), py * (My2 / My8)
    i0 = np.maximum(0, np.minimum(np.floor(u).astype(int), Mx2 - 2))
    j0 = np.maximum(0, np.minimum(np.floor(v).astype(int), My2 - 2))
    fu, fv = u - i0, v - j0
    i1, j1 = np.minimum(i0 + 1, Mx2 - 1), np.minimum(j0 + 1, My2 - 1)
    a, b = img2[j0][:, i0], img2[j0][:, i1]
    c, d = img2[j1][:, i0], img2[j1][:, i1]
    df = (1 - fv)[:, None] * ((1 - fu) * a + fu * b) + fv[:, None] * ((1 - fu) * c + fu * d)
    got = planes.cpu().numpy()
    m = mean.item()
    assert np.abs(got[4] - df).max() <= 2e-7
    assert np.abs(got[0] - (df - m) * 20.0).max() <= 5e-6
    assert np.array_equal(got[1], -got[0])
    assert np.all(got[2] == np.float32(0.25)) and np.all(got[3] == np.float32(m))
    packed = nn.pack(planes[:4].view(4, 1, Hp, Wp), 16).float().cpu().numpy()[0]
    want = np.zeros((Hp, Wp, 16), dtype=np.float32)
    want[..., :4] = NO.bf16_round(np.moveaxis(got[:4], 0, -1))
    assert np.array_equal(packed, want)
    # the corrected image: base + channel 0 of the prediction x scale, FP64, on the image's
    # My8 x Mx8 block of the padded grid
    pred = torch.from_numpy(rng.standard_normal((Hp, Wp, 16)).astype(np.float32)).cuda()
    out = torch.empty((My8, Mx8), dtype=torch.float64, device="cuda")
    nn.apply_correction(planes[4], pred, Mx8, My8, 0.01, out)
    want = got[4][:My8, :Mx8].astype(np.float64) + \
        pred.cpu().numpy()[:My8, :Mx8, 0].astype(np.float64) * np.float64(np.float32(0.01))
    assert np.abs(out.cpu().numpy() - want).max() <= 1e-15
