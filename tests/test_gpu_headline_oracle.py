"""The benchmark's own configurations against the oracle, whole images.

Each workload the bench reports is imaged through the C ABI on the GPU and compared
with the oracle (the FP64 C restatement of computeD2BI_img, on every host core):

* the 1.2M-atom screw + voids image (566 x 566 x 240 voxels), FP32 and FP64 paths,
  all 566 x 566 pixels;
* the 128k-atom void cell with -density, dark field, bright field and both blurred
  at 2.5 A, whole images;
* the tilt x precession x g sweep (41 tilts x 16 precession angles x 3 g, one batch
  on the GPU): the mid-series tilt of each g on a band of 24 pixel rows;
* the largest of the 256 uneven cells, imaged in the 256-cell FP32 batch, whole.

Bars: FP64 max |dI| <= 1e-12 (the reference's operation order; only exp, sin, cos
and hypot may differ in the last ulp), FP32 max |dI| <= 1e-4 and RMS <= 2e-5 (the
FP32 + FP64-phase path's bar).
"""
import os

import numpy as np
import pytest
import torch

from oracle import stem_oracle as O
from simulated_tem_gb300 import _lib, imaging, synth

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-4
FP32_RMS = 2e-5
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


def _oracle_state(cell, g=(1, 1, 0), sg=0.01, density=False, n_tomo=1, step=0):
    args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), g, sg=sg, xi0=103.9, xig=207.5, density=density,
                       nTomo=n_tomo, tomoAngle=20.0)
    so, xo, aperpx = O.setup(args, cell.pos, nn=step)
    return so, xo, aperpx


def _check(got, want, tol, rms=None):
    d = got - want
    assert np.abs(d).max() <= tol, float(np.abs(d).max())
    if rms is not None:
        assert np.sqrt((d ** 2).mean()) <= rms


def test_1p2m_image_whole_vs_oracle(ctx):
    """The headline image: FP32 and FP64 GPU images against the oracle on all 566 x 566 pixels."""
    cell = synth.screw_cell_1p2m()
    t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.01,
                                     xi0=103.9, xig=207.5, V=200.0, M=(4, 4))
    G, aa = t.image_geometry(len(x))
    assert (G.Mx, G.My, G.Mz) == (566, 566, 240)
    img32 = ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32 | _lib.ST_FLAG_STATS)
    st32 = ctx.stats()
    img64 = ctx.image(G, x, aa, flags=_lib.ST_FLAG_STATS)
    st64 = ctx.stats()
    so, xo, _ = _oracle_state(cell)
    assert np.array_equal(xo, x)
    Go, aao = O.geometry(so, len(xo))
    want, ost = O.patch_image(Go, aao, xo, nthreads=THREADS)
    assert want.max() > 0
    _check(img64, want, FP64_TOL)
    _check(img32, want, FP32_TOL, FP32_RMS)
    # the same link cells and the same accepted pairs as the reference's loops
    assert st64.n_kept == ost.n_kept and st32.n_kept == ost.n_kept
    assert st64.n_accepted == ost.n_accepted
    assert abs(st32.n_accepted - ost.n_accepted) <= 1e-5 * ost.n_accepted  # FP32 distances: flips at the cutoff


def test_128k_density_df_bf_blur_vs_oracle(ctx):
    """The CPU-runnable configuration: 128k atoms, 8 voids, s_g = 0, -density; dark field,
    bright field (1 - DF) and both blurred at 2.5 A, whole images, FP64 and FP32."""
    cell = synth.void_cell_128k()
    t, x, aperpx = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.0,
                                          xi0=103.9, xig=207.5, V=200.0, M=(4, 4), density=True)
    G, aa = t.image_geometry(len(x))
    so, xo, aperpx_o = _oracle_state(cell, sg=0.0, density=True)
    assert np.array_equal(xo, x) and aperpx_o == aperpx
    Go, aao = O.geometry(so, len(xo))
    df_o, _ = O.patch_image(Go, aao, xo, nthreads=THREADS)
    tpx = 2.5 / aperpx
    want = {"df": df_o, "bf": 1.0 - df_o, "df_blur": O.gaussian_blur(df_o, tpx),
            "bf_blur": O.gaussian_blur(1.0 - df_o, tpx)}
    for flags, tol, rms in ((0, FP64_TOL, None), (_lib.ST_FLAG_FP32, FP32_TOL, FP32_RMS)):
        df = ctx.image(G, x, aa, flags=flags | _lib.ST_FLAG_AVERAGE)
        bf = ctx.image(G, x, aa, flags=flags | _lib.ST_FLAG_AVERAGE | _lib.ST_FLAG_BRIGHT)
        got = {"df": df, "bf": bf, "df_blur": ctx.blur(df, tpx), "bf_blur": ctx.blur(bf, tpx)}
        for k in want:
            _check(got[k], want[k], tol, rms)


def test_sweep_images_vs_oracle(ctx):
    """The 123-image sweep as the bench runs it (one FP32 batch, images averaged over 16
    precession angles): the mid-series tilt of each g against the oracle on 24 pixel rows."""
    cell = synth.screw_cell_1p2m()
    gs = ((1, 1, 0), (2, 0, 0), (2, 1, 1))
    d_x, specs, _ = imaging.d2bi_sweep(ctx, cell.a_super, synth.A0_FE, (0, 0, 1), gs, cell.pos, n_tomo=41,
                                       tomo_angle=20.0, prec_angle=0.005, n_prec=16, sg=0.01, xi0=103.9, xig=207.5)
    imgs = [torch.empty((G.My, G.Mx), dtype=torch.float64, device="cuda") for G, _ in specs]
    jobs = [(G, d_x.data_ptr(), d_x.shape[0], aa, im.data_ptr()) for (G, aa), im in zip(specs, imgs)]
    torch.cuda.synchronize()
    ctx.batch_device(jobs, _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for gi, g in enumerate(gs):
        k = gi * 41 + 20
        G, aa = specs[k]
        got = imgs[k].cpu().numpy().T
        so, xo, _ = _oracle_state(cell, g=g, n_tomo=41, step=20)
        assert np.array_equal(xo, d_x.cpu().numpy())
        Go, aao = O.geometry(so, len(xo), nPrec=16, precAngle=0.005)
        assert np.array_equal(aao, aa)
        mid = (G.iy0 + G.iy1) // 2
        lo, hi = mid - 12, mid + 12
        want, _ = O.patch_image(Go, aao, xo, rows=(lo, hi), nthreads=THREADS)
        want = want / 16
        assert want[:, lo:hi].max() > 0
        _check(got[:, lo:hi], want[:, lo:hi], FP32_TOL, FP32_RMS)


def test_largest_uneven_cell_vs_oracle(ctx):
    """The 256 uneven cells in one FP32 batch; the largest (the slowest image of the batch)
    against the oracle, whole."""
    cells = synth.uneven_cells()
    specs = []
    for cell, sg in cells:
        t, xw, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=sg,
                                          xi0=103.9, xig=207.5, V=200.0, M=(4, 4))
        G, aa = t.image_geometry(len(xw))
        specs.append((G, aa, xw))
    d_xs = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for _, _, x in specs]
    imgs = [torch.empty((G.My, G.Mx), dtype=torch.float64, device="cuda") for G, _, _ in specs]
    jobs = [(G, dx.data_ptr(), len(x), aa, im.data_ptr()) for (G, aa, x), dx, im in zip(specs, d_xs, imgs)]
    torch.cuda.synchronize()
    ctx.batch_device(jobs, _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    k = int(np.argmax([len(x) for _, _, x in specs]))
    cell, sg = cells[k]
    so, xo, _ = _oracle_state(cell, sg=sg)
    assert np.array_equal(xo, specs[k][2])
    Go, aao = O.geometry(so, len(xo))
    want, _ = O.patch_image(Go, aao, xo, nthreads=THREADS)
    _check(imgs[k].cpu().numpy().T, want, FP32_TOL, FP32_RMS)
