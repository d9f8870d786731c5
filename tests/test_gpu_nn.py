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
