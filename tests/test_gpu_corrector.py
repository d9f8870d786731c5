"""The learned corrector on the GPU: masked fine solves, gradients of the whole network
against the CPU oracle, what training gains over the interpolated coarse image, and the
fallback to the plain fine-grid solve."""
import numpy as np
import pytest

from oracle import nn_oracle as NO
from simulated_tem_gb300 import _lib, imaging, synth

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def C():
    from simulated_tem_gb300 import corrector
    return corrector


def _four_slices_fit(G):
    """Every step of four slices has home z cells rising by at most one, without a wrap
    (Lib_DynamicalTwoBeamImaging.f90:1878-1879 for the home cell of a slice)."""
    h = [(int(np.floor(G.ia_col[8] * (G.a_vox[8] * z - G.lc_delta[2]))) + 16 * G.Ez) % G.Ez for z in range(G.Mz)]
    for z0 in range(0, G.Mz, 4):
        s = h[z0:z0 + 4]
        if any(b < a for a, b in zip(s, s[1:])) or s[-1] - s[0] > 1:
            return False
    return True


@pytest.mark.parametrize("fp32", [False, True])
def test_masked_image_equals_full_on_its_tiles(ctx, fp32):
    """A tile-masked image equals the plain one on its tiles.  In FP64 the plain image
    marches four slices per step (its steps fit the ring) and the masked one two, so this
    also pins the four-slice FP64 march to the two-slice one, bit for bit."""
    cell = synth.small_cell(n=(12, 12, 6), seed=21, n_voids=1, radius=(4.0, 6.0), with_screw=True)
    t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.01, M=(6, 6))
    G, aa = t.image_geometry(len(x))
    assert _four_slices_fit(G)
    flags = _lib.ST_FLAG_FP32 if fp32 else 0
    full = ctx.image(G, x, aa, flags=flags)
    T = 16
    ntx, nty = (G.Mx + T - 1) // T, (G.My + T - 1) // T
    mask = (np.random.default_rng(2).random((nty, ntx)) < 0.4).astype(np.uint8)
    d_x = torch.from_numpy(x).cuda()
    img = torch.full((G.My, G.Mx), 3.0, dtype=torch.float64, device="cuda")
    d_mask = torch.from_numpy(mask).cuda()
    torch.cuda.synchronize()
    ctx.image_device_masked(G, d_x.data_ptr(), len(x), aa, flags, img.data_ptr(), d_mask.data_ptr(), T,
                            stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = img.cpu().numpy().T
    sel = np.kron(mask, np.ones((T, T), dtype=np.uint8))[:G.My, :G.Mx].T.astype(bool)
    assert np.array_equal(got[sel], full[sel])
    assert not got[~sel].any()


def test_network_gradients_match_oracle(C):
    """Loss and every parameter gradient of the U-Net (BF16 activations, tensor-core
    convolutions) against the float64 oracle on a 16 x 16 input."""
    from simulated_tem_gb300 import nn as N
    model = C.UNet(seed=3, head_std=0.1)
    rng = np.random.default_rng(4)
    x = np.zeros((2, 16, 16, C.IN_C), dtype=np.float32)
    x[..., :3] = rng.standard_normal((2, 16, 16, 3))
    x = NO.bf16_round(x)
    tgt = rng.standard_normal((2, 16, 16)).astype(np.float32)
    xd = torch.from_numpy(x).to(torch.bfloat16).cuda()
    out = model.forward(xd, keep=True)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    g = torch.empty((2, 16, 16, C.OUT_C), dtype=torch.bfloat16, device="cuda")
    N.mse(out, torch.from_numpy(tgt).cuda(), g, loss)
    model.backward(g)
    torch.cuda.synchronize()
    assert N.last_kernel_error() == 0
    P = {}
    for name, cin, cout, taps, _ in model.specs:
        P[name + ".w"] = model.weight(name).float().cpu().numpy().astype(np.float64)
        P[name + ".b"] = model.bias(name).cpu().numpy().astype(np.float64)
    # the oracle with BF16 rounding where the GPU stores BF16: only FP32 accumulation order
    # (and the rare BF16 rounding it flips) differs
    want_loss, G = NO.unet_loss_grads(P, x, tgt, C.CH, bf16=True)
    assert abs(loss.item() - want_loss) <= 1e-3 * want_loss
    for name, cin, cout, taps, _ in model.specs:
        for kind, got in (("w", model.gweight(name)), ("b", model.gbias(name))):
            got = got.cpu().numpy().astype(np.float64).ravel()
            want = G[name + "." + kind].ravel()
            rel = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-30)
            assert rel <= 1e-2, (name, kind, rel)
    # and the float64 network, as a sanity bound: BF16 storage of ~30 tensors on the way
    # moves the deepest layers' gradients by up to ~15 % (measured), the loss by < 2 %
    want_loss64, G64 = NO.unet_loss_grads(P, x, tgt, C.CH)
    assert abs(loss.item() - want_loss64) <= 2e-2 * want_loss64
    for name, cin, cout, taps, _ in model.specs:
        got = model.gweight(name).cpu().numpy().astype(np.float64).ravel()
        want = G64[name + ".w"].ravel()
        assert np.linalg.norm(got - want) <= 0.3 * np.linalg.norm(want), name


def _cells(n, seed, nxy=24, nz=40):
    """Small bcc Fe cells, 40 lattice cells (115 A) thick so that the images have contrast."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        cell = synth.make_cell(nxy, nxy, nz, int(rng.integers(1 << 30)), n_voids=int(rng.integers(1, 5)),
                               void_radius=(4.0, 10.0), with_screw=bool(i % 2))
        out.append(cell)
    return out


def _pairs(ctx, C, cells, n_sg, seed):
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    for cell in cells:
        a, b = C.make_pairs(ctx, cell, list(rng.uniform(-0.02, 0.02, n_sg)), 128, 2, rng)
        xs.append(a)
        ys.append(b)
    return np.concatenate(xs), np.concatenate(ys)


def test_training_beats_interpolation(ctx, C):
    """Trained on pairs from twelve small cells (the M = 2 and M = 8 solves of this
    library), the corrector's image of held-out cells is closer to the M = 8 solve than the
    interpolated M = 2 image: what the network gains over the method without it."""
    xtr, ytr = _pairs(ctx, C, _cells(12, 6), 6, 1)
    xte, yte = _pairs(ctx, C, _cells(3, 99), 3, 2)
    model = C.UNet(seed=1)
    before = C.evaluate(model, xte, yte)
    trainer = C.Trainer(model, xtr, ytr, batch=4)
    trainer.run(2000, lr=3e-3, lr_end=1e-4)
    after = C.evaluate(model, xte, yte)
    from simulated_tem_gb300 import nn as N
    assert N.last_kernel_error() == 0
    # training is deterministic (gradients summed in a fixed order); measured on a GB300:
    # 0.919 of the interpolated coarse image's RMS error
    assert after["rms_corrected"] < 0.95 * after["rms_uncorrected"], (before, after)
    assert after["rms_corrected"] < before["rms_corrected"]


def test_fallback_reproduces_the_fine_solve(ctx, C):
    """With tau = 0 every tile falls back: the image is the plain M = 8 solve exactly; with an
    infinite tau only the border ring of tiles does (with the ring always recomputed)."""
    cell = _cells(1, 9, nxy=16, nz=12)[0]
    t2, x = C.condition(cell, 2, 0.01)
    t8, _ = C.condition(cell, 8, 0.01)
    G8, aa8 = t8.image_geometry(len(x))
    fine = ctx.image(G8, x, aa8, flags=_lib.ST_FLAG_FP32)
    d_x = torch.from_numpy(x).cuda()
    model = C.UNet(seed=2)
    img, nflag, ntiles = C.CorrectedImager(model, ctx, tile=32, tau=0.0).image(t2, t8, d_x, len(x), 0.01)
    torch.cuda.synchronize()
    assert nflag == ntiles
    assert np.array_equal(img.cpu().numpy().T, fine)
    img, nflag, _ = C.CorrectedImager(model, ctx, tile=32, tau=np.inf).image(t2, t8, d_x, len(x), 0.01)
    ntx, nty = (G8.Mx + 31) // 32, (G8.My + 31) // 32
    assert nflag == 2 * (ntx + nty) - 4
    got = img.cpu().numpy().T
    assert np.isfinite(got).all()
    assert np.array_equal(got[:32, :], fine[:32, :]) and np.array_equal(got[:, -1], fine[:, -1])
