"""The corrector's CPU oracle (oracle/nn_oracle.py) against finite differences and
direct definitions, so that it can check the GPU kernels' gradients."""
import numpy as np

from oracle import nn_oracle as NO

CH = (8, 8, 16, 16)


def _params(rng):
    c = CH
    specs = [("enc0a", 16, c[0], 9), ("enc0b", c[0], c[0], 9), ("enc1a", c[0], c[1], 9), ("enc1b", c[1], c[1], 9),
             ("enc2a", c[1], c[2], 9), ("enc2b", c[2], c[2], 9), ("bota", c[2], c[3], 9), ("botb", c[3], c[3], 9),
             ("dec2a", c[3] + c[2], c[2], 9), ("dec2b", c[2], c[2], 9), ("dec1a", c[2] + c[1], c[1], 9),
             ("dec1b", c[1], c[1], 9), ("dec0a", c[1] + c[0], c[0], 9), ("dec0b", c[0], c[0], 9),
             ("head", c[0], 16, 1)]
    P = {}
    for n, ci, co, t in specs:
        P[n + ".w"] = rng.standard_normal((co, t, ci)) * np.sqrt(2.0 / (t * ci))
        P[n + ".b"] = rng.standard_normal(co) * 0.1
    return P


def test_network_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    P = _params(rng)
    x = rng.standard_normal((1, 8, 8, 16))
    tgt = rng.standard_normal((1, 8, 8))
    _, G = NO.unet_loss_grads(P, x, tgt, CH)
    for name in ["enc0a.w", "enc1b.w", "bota.b", "dec2a.w", "dec1a.w", "dec0b.b", "head.w", "head.b"]:
        for _ in range(3):
            idx = tuple(int(rng.integers(0, s)) for s in P[name].shape)
            if name.startswith("head"):
                idx = (0,) + idx[1:]  # channel 0 carries the loss
            eps = 1e-6
            P[name][idx] += eps
            lp, _ = NO.unet_loss_grads(P, x, tgt, CH)
            P[name][idx] -= 2 * eps
            lm, _ = NO.unet_loss_grads(P, x, tgt, CH)
            P[name][idx] += eps
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - G[name][idx]) <= 1e-6 + 1e-5 * abs(fd), (name, idx, fd, G[name][idx])


def test_conv_oracle_matches_loops():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((1, 5, 6, 3))
    w = rng.standard_normal((4, 9, 3))
    y = NO.conv2d(x, w)
    want = np.zeros((1, 5, 6, 4))
    for yy in range(5):
        for xx in range(6):
            for t in range(9):
                dy, dx = t // 3 - 1, t % 3 - 1
                if 0 <= yy + dy < 5 and 0 <= xx + dx < 6:
                    want[0, yy, xx] += w[:, t, :] @ x[0, yy + dy, xx + dx]
    assert np.allclose(y, want)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-30, 3.0e38], dtype=np.float32)
    r = NO.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0 + 4 * 2 ** -8)
    assert r[3] == -2.5
    assert np.array_equal(NO.from_bf16_bits(NO.bf16_bits(v)), r)
