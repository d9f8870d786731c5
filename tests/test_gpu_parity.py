"""Parity of the CUDA path (through the C ABI) with the oracle.

Bars: FP64 path max |dI| <= 1e-12 against the oracle (same accept set, same
summation order; only exp/sin/cos/hypot may differ in the last ulp); FP32
path max |dI| <= 1e-4 (the precision target of the FP32 + FP64-phase path);
binning counts and accepted-pair counts identical; the blur identical to the
last bit.
"""
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import _lib, imaging, synth
from tests import golden_data

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


def setup_both(cell, a0=synth.A0_FE, k=(0, 0, 1), g=(1, 1, 0), **kw):
    m = dict(kw)
    t, xw, _ = imaging.d2bi_condition(cell.a_super, a0, k, g, cell.pos, **m)
    ok = {"sg": "sg", "R": "R", "U": "U", "d": "d", "xi0": "xi0", "xig": "xig", "density": "density"}
    args = O.make_args(cell.a_super, a0, k, g, **{ok[kk]: v for kk, v in kw.items() if kk in ok})
    so, xo, _ = O.setup(args, cell.pos)
    assert np.array_equal(xw, xo)
    return t, so, xw


def oracle_patch(so, x, n_prec, prec_angle, nprocs=1, jj=0):
    G, aa = O.geometry(so, len(x), nPrec=n_prec, precAngle=prec_angle, nProcs=nprocs, jj=jj)
    img, st = O.patch_image(G, aa, x, nthreads=8)
    return img, st


CELLS = {
    "screw+void": dict(n=(10, 10, 8), seed=5, n_voids=1, radius=(4.0, 6.0), with_screw=True),
    "voids": dict(n=(9, 11, 7), seed=6, n_voids=3, radius=(3.0, 5.0), with_screw=False),
}


@pytest.mark.parametrize("cell_name", sorted(CELLS))
@pytest.mark.parametrize("density", [False, True])
@pytest.mark.parametrize("sg", [0.0, 0.01])
def test_fp64_matches_oracle(ctx, cell_name, density, sg):
    cell = synth.small_cell(**CELLS[cell_name])
    t, so, x = setup_both(cell, sg=sg, density=density)
    G, aa = t.image_geometry(len(x))
    got = ctx.image(G, x, aa, flags=_lib.ST_FLAG_STATS)
    st = ctx.stats()
    want, ost = oracle_patch(so, x, 1, 0.005)
    assert np.abs(got - want).max() <= FP64_TOL
    assert st.n_kept == ost.n_kept
    assert st.n_accepted == ost.n_accepted
    assert st.max_cell_count == ost.max_cell_count


@pytest.mark.parametrize("cell_name", sorted(CELLS))
@pytest.mark.parametrize("density", [False, True])
def test_fp32_matches_oracle(ctx, cell_name, density):
    cell = synth.small_cell(**CELLS[cell_name])
    t, so, x = setup_both(cell, sg=0.01, density=density)
    G, aa = t.image_geometry(len(x))
    got = ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32 | _lib.ST_FLAG_STATS)
    st = ctx.stats()
    want, ost = oracle_patch(so, x, 1, 0.005)
    d = got - want
    assert np.abs(d).max() <= FP32_TOL
    assert np.sqrt((d ** 2).mean()) <= FP32_TOL / 5
    # the FP32 path's binning assigns cells exactly like the reference
    assert st.n_kept == ost.n_kept and st.max_cell_count == ost.max_cell_count


@pytest.mark.parametrize("n_prec,fp32", [(3, False), (6, False), (5, True), (17, True)])
def test_precession_passes(ctx, n_prec, fp32):
    """Precession: one phase field, n_prec integrations (the FP64 kernel runs 4 per
    pass, the FP32 kernel 16 per pass), averaged (ST_FLAG_AVERAGE)."""
    cell = synth.small_cell(**CELLS["screw+void"])
    t, so, x = setup_both(cell, sg=0.01, density=True)
    G, aa = t.image_geometry(len(x), prec_angle=0.005, n_prec=n_prec)
    flags = _lib.ST_FLAG_AVERAGE | (_lib.ST_FLAG_FP32 if fp32 else 0)
    got = ctx.image(G, x, aa, flags=flags)
    want, _ = oracle_patch(so, x, n_prec, 0.005)
    want = want / n_prec
    assert np.abs(got - want).max() <= (FP32_TOL if fp32 else FP64_TOL)
    # tilts around the cone: s_g(phi) = s_g(2 pi - phi), so the angles come in equal pairs
    assert len(set(np.round(aa, 12))) >= (n_prec + 1) // 2


def test_bright_field_and_average(ctx):
    cell = synth.small_cell(**CELLS["voids"])
    t, so, x = setup_both(cell, sg=0.0)
    G, aa = t.image_geometry(len(x), n_prec=2)
    raw = ctx.image(G, x, aa)
    bf = ctx.image(G, x, aa, flags=_lib.ST_FLAG_AVERAGE | _lib.ST_FLAG_BRIGHT)
    assert np.array_equal(bf, 1.0 - raw / 2)


@pytest.mark.parametrize("nprocs", [2, 3, 4])
def test_patches_match_oracle(ctx, nprocs):
    """The reference's MPI patch split: each process images its patch; the sum of the
    zero-padded patch images is the image (MPI_Reduce SUM)."""
    cell = synth.small_cell(**CELLS["screw+void"])
    t, so, x = setup_both(cell, sg=0.01, density=True)
    total = None
    for jj in range(nprocs):
        G, aa = t.image_geometry(len(x), nprocs=nprocs, jj=jj)
        got = ctx.image(G, x, aa)
        want, _ = oracle_patch(so, x, 1, 0.005, nprocs=nprocs, jj=jj)
        assert np.abs(got - want).max() <= FP64_TOL
        outside = np.ones_like(got, dtype=bool)
        outside[G.ix0:G.ix1, G.iy0:G.iy1] = False
        assert not got[outside].any()
        total = got if total is None else total + got
    G1, aa1 = t.image_geometry(len(x))
    full = ctx.image(G1, x, aa1)
    # different patches shift the link-cell origin: equal to rounding, not to the bit
    assert np.abs(total - full).max() < 1e-9


def test_full_size_workload(ctx):
    """The benchmark's image at full size: the 1.2M-atom screw + voids cell, g = [110],
    s_g = 0.01, M = 4 (566 x 566 x 240 voxels).  The FP32 path within 1e-4 of the FP64 path
    over the whole image; repeated FP32 images identical bit for bit; the FP64 path equal to
    the oracle on 16 middle rows (the oracle's row range keeps the CPU time to seconds)."""
    cell = synth.screw_cell_1p2m()
    t, so, x = setup_both(cell, sg=0.01, xi0=103.9, xig=207.5)
    G, aa = t.image_geometry(len(x))
    assert (G.Mx, G.My, G.Mz) == (566, 566, 240)
    img64 = ctx.image(G, x, aa)
    img32 = ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
    again = ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
    assert np.isfinite(img64).all() and img64.max() > 0
    assert np.abs(img32 - img64).max() <= FP32_TOL
    assert np.array_equal(img32, again)
    Go, aao = O.geometry(so, len(x))
    lo, hi = 275, 291
    want, _ = O.patch_image(Go, aao, x, rows=(lo, hi), nthreads=8)
    assert np.abs(img64[:, lo:hi] - want[:, lo:hi]).max() <= FP64_TOL
    assert want[:, lo:hi].max() > 0


def test_w_loop_golden_on_gpu(ctx):
    g = golden_data.w_loop()
    cell = synth.Cell(g["a_super"], g["pos"])
    t, so, x = setup_both(cell, a0=3.1652, g=(2, 0, 0), R=g["RU"], U=np.eye(3), d=g["d"], xi0=g["xi0"],
                          xig=g["xig"])
    img64 = t.compute_d2bi_img(ctx, x)
    img32 = t.compute_d2bi_img(ctx, x, flags=_lib.ST_FLAG_FP32)
    want, _ = oracle_patch(so, x, 1, 0.005)
    assert np.abs(img64 - want).max() <= FP64_TOL
    assert np.abs(img32 - want).max() <= FP32_TOL
    assert np.abs(img64 - g["img"]).max() < 2e-4


def test_blur_matches_oracle(ctx):
    g = golden_data.w_loop()
    for t in (3.1446, 0.7, 12.0):
        got = ctx.blur(g["img"], t)
        want = O.gaussian_blur(g["img"], t)
        assert np.array_equal(got, want)
    rect = np.random.default_rng(1).random((37, 53))
    assert np.array_equal(ctx.blur(rect, 2.2), O.gaussian_blur(rect, 2.2))


def test_empty_input(ctx):
    """No atoms: every voxel is void (x = 0), so no diffracted intensity."""
    cell = synth.small_cell(**CELLS["voids"])
    t, so, x = setup_both(cell, sg=0.01, density=True)
    G, aa = t.image_geometry(0)
    got = ctx.image(G, np.zeros((0, 3)), aa)
    want, _ = oracle_patch(so, np.zeros((0, 3)), 1, 0.005)
    assert np.array_equal(got, want)
    assert not got.any()


def test_ldx_fourteen(ctx):
    """d2bi passes x(1:14, nAtoms) when the input had fewer than 14 columns."""
    cell = synth.small_cell(**CELLS["voids"])
    t, so, x = setup_both(cell, sg=0.01)
    x14 = np.zeros((len(x), 14))
    x14[:, :3] = x
    x14[:, 3:] = 7.0
    G, aa = t.image_geometry(len(x))
    assert np.array_equal(ctx.image(G, x14, aa), ctx.image(G, x, aa))


def test_errors_are_reported(ctx):
    cell = synth.small_cell(**CELLS["voids"])
    t, so, x = setup_both(cell, sg=0.01)
    G, aa = t.image_geometry(len(x))
    with pytest.raises(_lib.StemError) as e:
        ctx.image(G, x, np.zeros(0))
    assert e.value.code == _lib.ST_ERR_ARG
    G2, _ = t.image_geometry(len(x))
    G2.a_vox[1] = 1e-3  # not a cuboid voxel
    with pytest.raises(_lib.StemError) as e:
        ctx.image(G2, x, aa)
    assert e.value.code == _lib.ST_ERR_ARG and "cuboid" in str(e.value)
    G3, _ = t.image_geometry(len(x))
    G3.nMax0 = 1  # the reference stops once a cell needs more than 16 x nMax0 slots
    dense = np.concatenate([x] * 20)
    with pytest.raises(_lib.StemError) as e:
        ctx.image(G3, dense, aa)
    assert e.value.code == _lib.ST_ERR_CAPACITY
    # the context stays usable
    assert np.isfinite(ctx.image(G, x, aa)).all()


def _general_fp32_context():
    import os
    old = os.environ.get("STEM_FP32_KERNEL")
    os.environ["STEM_FP32_KERNEL"] = "general"
    try:
        return imaging.Context(0)
    finally:
        if old is None:
            del os.environ["STEM_FP32_KERNEL"]
        else:
            os.environ["STEM_FP32_KERNEL"] = old


@pytest.mark.parametrize("density", [False, True])
def test_fp32_ring_and_general_kernels_agree(ctx, density):
    """The slab-ring FP32 kernel and the general FP32 kernel compute the same image."""
    cell = synth.small_cell(**CELLS["screw+void"])
    t, so, x = setup_both(cell, sg=0.01, density=density)
    G, aa = t.image_geometry(len(x), n_prec=3)
    ring = ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32 | _lib.ST_FLAG_STATS)
    assert ctx.stats().column_kernel == 2
    gctx = _general_fp32_context()
    try:
        gen = gctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32 | _lib.ST_FLAG_STATS)
        assert gctx.stats().column_kernel == 1
    finally:
        gctx.close()
    want, _ = oracle_patch(so, x, 3, 0.005)
    assert np.abs(ring - want).max() <= FP32_TOL
    assert np.abs(gen - want).max() <= FP32_TOL
    assert np.abs(ring - gen).max() <= 2e-5


def test_fp32_ring_overflow_falls_back(ctx):
    """Sixteen copies of every atom overfill even 256-atom slabs: the image is recomputed by
    the general kernel and still matches the oracle."""
    cell = synth.small_cell(**CELLS["voids"])
    dense = synth.Cell(cell.a_super, np.concatenate([cell.pos] * 16))
    t, so, x = setup_both(dense, sg=0.01)
    G, aa = t.image_geometry(len(x))
    c = imaging.Context(0)
    try:
        got = c.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
        assert c.stats().column_kernel == 1
    finally:
        c.close()
    want, _ = oracle_patch(so, x, 1, 0.005)
    assert np.abs(got - want).max() <= FP32_TOL


def test_fp32_ring_big_slabs(ctx):
    """Three copies of every atom overfill 128-atom slabs: the ring kernel reruns with
    256-atom slabs, and the context keeps them for the next image of that kind."""
    cell = synth.small_cell(**CELLS["voids"])
    dense = synth.Cell(cell.a_super, np.concatenate([cell.pos] * 3))
    t, so, x = setup_both(dense, sg=0.01)
    G, aa = t.image_geometry(len(x))
    c = imaging.Context(0)
    try:
        got = c.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
        assert c.stats().column_kernel == 2
        again = c.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
        assert c.stats().column_kernel == 2
        assert np.array_equal(again, got)
    finally:
        c.close()
    want, _ = oracle_patch(so, x, 1, 0.005)
    assert np.abs(got - want).max() <= FP32_TOL


def _context_with(env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return imaging.Context(0)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def test_fp32_ring_slab_capacities_agree(ctx):
    """The slab ring's staging capacity (128, 192, 256 atoms) changes neither which
    candidates are tested nor their order: the three give the same image bit for bit;
    two copies of every atom need the 192-atom tier or more."""
    cell = synth.small_cell(**CELLS["screw+void"])
    t, so, x = setup_both(cell, sg=0.01)
    G, aa = t.image_geometry(len(x), n_prec=2)
    imgs = {}
    for slabs in ("128", "192", "256"):
        c = _context_with({"STEM_RING_SLABS": slabs})
        try:
            imgs[slabs] = c.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
            assert c.stats().column_kernel == 2 and c.stats().ring_slab_atoms == int(slabs)
        finally:
            c.close()
    assert np.array_equal(imgs["128"], imgs["192"]) and np.array_equal(imgs["128"], imgs["256"])
    dense = synth.Cell(cell.a_super, np.concatenate([cell.pos] * 2))
    t2, so2, x2 = setup_both(dense, sg=0.01)
    G2, aa2 = t2.image_geometry(len(x2))
    c = imaging.Context(0)
    try:
        got = c.image(G2, x2, aa2, flags=_lib.ST_FLAG_FP32)
        assert c.stats().column_kernel == 2 and c.stats().ring_slab_atoms in (192, 256)
    finally:
        c.close()
    want, _ = oracle_patch(so2, x2, 1, 0.005)
    assert np.abs(got - want).max() <= FP32_TOL


@pytest.mark.parametrize("short", [0.9999997, 0.8, 0.55])
def test_fp32_ring_truncated_z_search(ctx, short):
    """z link cells shorter than 3 sigma (a z voxel smaller than the in-plane one: deltaM
    comes from the in-plane side, Lib_DynamicalTwoBeamImaging.f90:1753-1773): the reference
    searches only the 27 cells around each voxel's home cell.  The slab ring applies that
    rule slab by slab; it agrees with the general FP32 kernel (which tests cell offsets) and
    with the FP64 path, which follows the reference's 27-cell search."""
    cell = synth.small_cell(**CELLS["screw+void"])
    t, so, x = setup_both(cell, sg=0.01)
    G, aa = t.image_geometry(len(x))
    # z voxels `short` x the cell height 3 sigma / 6: six voxels per z cell
    G.Ez = max(3, G.Ez)
    G.Mz = 6 * G.Ez
    G.a_vox[8] = short * G.sigma / 2
    G.a_col[8] = G.Mz * G.a_vox[8] / G.Ez
    G.ia_col[8] = 1 / G.a_col[8]
    G.deltaz = G.a_vox[8]
    assert G.a_col[8] < 3 * G.sigma
    ring = ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
    assert ctx.stats().column_kernel == 2
    gctx = _general_fp32_context()
    try:
        gen = gctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
        assert gctx.stats().column_kernel == 1
    finally:
        gctx.close()
    f64 = ctx.image(G, x, aa, flags=0)
    assert np.abs(ring - gen).max() <= 2e-5
    assert np.abs(ring - f64).max() <= FP32_TOL


@pytest.mark.parametrize("n,M", [((10, 10, 7), (4, 5)), ((10, 10, 6), (4, 3)), ((10, 10, 7), (4, 3))])
def test_fp64_uneven_slice_counts_match_oracle(ctx, n, M):
    """The plain FP64 path with 35, 18 and 21 slices per column (3, 2 and 1 past a multiple
    of four: the four-slice march ends on a partial step; odd counts also leave the last
    interval to the integrator's rule) against the oracle, counts included."""
    cell = synth.small_cell(n=n, seed=7, n_voids=1, radius=(3.0, 5.0), with_screw=True)
    t, xw, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.01, M=M)
    args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), sg=0.01, M=M)
    so, xo, _ = O.setup(args, cell.pos)
    assert np.array_equal(xw, xo)
    G, aa = t.image_geometry(len(xw))
    assert G.Mz % 4 != 0
    got = ctx.image(G, xw, aa, flags=_lib.ST_FLAG_STATS)
    st = ctx.stats()
    assert st.column_kernel == 4  # the FP64 slab ring
    want, ost = oracle_patch(so, xw, 1, 0.005)
    assert np.abs(got - want).max() <= FP64_TOL
    assert st.n_kept == ost.n_kept and st.n_accepted == ost.n_accepted
