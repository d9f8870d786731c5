"""Batches through st_batch_device.

A batch runs one binning pass over the candidates of all its images and, on
the FP32 path, one persistent column launch over the warp tiles of all its
images.  Every image of a batch must equal, to the last bit, the image the
single-image entry point makes for the same job (same kernels, same
summation order per voxel), and must match the oracle to the path's bar.
"""
import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import _lib, imaging, synth

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


def _condition(cell, g=(1, 1, 0), n_tomo=1, step=0, **kw):
    t, xw, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), g, cell.pos, n_tomo=n_tomo,
                                      tomo_step=step, **kw)
    args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), g, nTomo=n_tomo,
                       **{k: v for k, v in kw.items() if k in ("sg", "density")})
    so, xo, _ = O.setup(args, cell.pos, nn=step)
    assert np.array_equal(xw, xo)
    return t, so, xw


def _batch(ctx, specs, flags):
    """specs: (geom, aa, x) per job; x arrays with the same id share one device buffer."""
    dev, imgs, jobs = {}, [], []
    for G, aa, x in specs:
        if id(x) not in dev:
            dev[id(x)] = torch.from_numpy(np.ascontiguousarray(x)).to("cuda") if len(x) else \
                torch.zeros(3, dtype=torch.float64, device="cuda")
        im = torch.full((G.My, G.Mx), 7.0, dtype=torch.float64, device="cuda")  # overwritten by the batch
        imgs.append(im)
        jobs.append((G, dev[id(x)].data_ptr(), len(x), aa, im.data_ptr()))
    torch.cuda.synchronize()
    ctx.batch_device(jobs, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return [im.cpu().numpy().T for im in imgs]


def _mixed_specs(fp32):
    """Images of different cells, sizes, g-vectors, density settings, precession counts and patches."""
    sv = synth.small_cell(n=(10, 10, 8), seed=5, n_voids=1, radius=(4.0, 6.0), with_screw=True)
    vo = synth.small_cell(n=(9, 11, 7), seed=6, n_voids=3, radius=(3.0, 5.0), with_screw=False)
    specs, oracles = [], []
    t, so, x = _condition(sv, sg=0.01, density=True)
    G, aa = t.image_geometry(len(x), n_prec=3)
    specs.append((G, aa, x)), oracles.append((so, x, 3, 1, 0))
    t, so, x2 = _condition(vo, sg=0.0)
    G, aa = t.image_geometry(len(x2))
    specs.append((G, aa, x2)), oracles.append((so, x2, 1, 1, 0))
    t, so, x3 = _condition(sv, g=(2, 0, 0), sg=-0.005)
    n_prec = 17 if fp32 else 6  # more angles than one pass of the column kernel holds
    G, aa = t.image_geometry(len(x3), n_prec=n_prec)
    specs.append((G, aa, x3)), oracles.append((so, x3, n_prec, 1, 0))
    t, so, x4 = _condition(vo, sg=0.01, density=True)
    G, aa = t.image_geometry(len(x4), nprocs=3, jj=1)
    specs.append((G, aa, x4)), oracles.append((so, x4, 1, 3, 1))
    G, aa = t.image_geometry(0)
    empty = np.zeros((0, 3))
    specs.append((G, aa, empty)), oracles.append((so, empty, 1, 1, 0))
    return specs, oracles


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("average", [False, True])
def test_mixed_batch_equals_single_images(ctx, fp32, average):
    flags = (_lib.ST_FLAG_FP32 if fp32 else 0) | (_lib.ST_FLAG_AVERAGE if average else 0)
    specs, oracles = _mixed_specs(fp32)
    got = _batch(ctx, specs, flags | _lib.ST_FLAG_STATS)
    st = ctx.stats()
    if fp32:
        assert st.column_kernel == 2  # one persistent slab-ring launch per pass
    n_kept = 0
    for (G, aa, x), img, (so, xo, n_prec, nprocs, jj) in zip(specs, got, oracles):
        single = ctx.image(G, x, aa, flags=flags | _lib.ST_FLAG_STATS)
        n_kept += ctx.stats().n_kept
        assert np.array_equal(img, single)
        Go, aao = O.geometry(so, len(xo), nPrec=n_prec, precAngle=0.005, nProcs=nprocs, jj=jj)
        want, _ = O.patch_image(Go, aao, xo, nthreads=8)
        if average:
            want = want.copy()
            want[Go.ix0:Go.ix1, Go.iy0:Go.iy1] /= n_prec
        assert np.abs(img - want).max() <= (FP32_TOL if fp32 else FP64_TOL)
    assert st.n_kept == n_kept


@pytest.mark.parametrize("fp32", [False, True])
def test_tomography_series_shares_atoms(ctx, fp32):
    """A tilt series: five tomography tilts of one cell image the same device atoms."""
    cell = synth.small_cell(n=(10, 10, 8), seed=5, n_voids=1, radius=(4.0, 6.0), with_screw=True)
    specs, oracles = [], []
    x0 = None
    for step in range(5):
        t, so, x = _condition(cell, n_tomo=5, step=step, sg=0.01, density=True)
        x0 = x if x0 is None else x0
        assert np.array_equal(x, x0)
        G, aa = t.image_geometry(len(x0), n_prec=2)
        specs.append((G, aa, x0))
        oracles.append(so)
    flags = _lib.ST_FLAG_FP32 if fp32 else 0
    got = _batch(ctx, specs, flags)
    for (G, aa, x), img, so in zip(specs, got, oracles):
        assert np.array_equal(img, ctx.image(G, x, aa, flags=flags))
        Go, aao = O.geometry(so, len(x), nPrec=2, precAngle=0.005)
        want, _ = O.patch_image(Go, aao, x, nthreads=8)
        assert np.abs(img - want).max() <= (FP32_TOL if fp32 else FP64_TOL)
    assert not np.array_equal(got[0], got[2])  # the tilts give different images


def test_uneven_cells_batch(ctx):
    """Independent cells of 0.6k to 60k atoms and different shapes in one FP32 batch."""
    cells = synth.uneven_cells(count=12, lo=8_000, hi=60_000)  # voids leave 637 to 57k atoms
    specs = []
    for cell, sg in cells:
        t, xw, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=sg)
        G, aa = t.image_geometry(len(xw))
        specs.append((G, aa, xw))
    assert len({(G.Mx, G.My, G.Mz) for G, _, _ in specs}) > 6
    got = _batch(ctx, specs, _lib.ST_FLAG_FP32)
    for (G, aa, x), img in zip(specs, got):
        assert np.array_equal(img, ctx.image(G, x, aa, flags=_lib.ST_FLAG_FP32))
    # the smallest cell against the oracle
    k = int(np.argmin([cell.n_atoms for cell, _ in cells]))
    cell, sg = cells[k]
    args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), sg=sg)
    so, xo, _ = O.setup(args, cell.pos)
    assert np.array_equal(xo, specs[k][2])
    Go, aao = O.geometry(so, len(xo))
    want, _ = O.patch_image(Go, aao, xo, nthreads=8)
    assert np.abs(got[k] - want).max() <= FP32_TOL


def test_batch_errors(ctx):
    cell = synth.small_cell()
    t, so, x = _condition(cell, sg=0.01)
    G, aa = t.image_geometry(len(x))
    xd = torch.from_numpy(x).to("cuda")
    im = torch.zeros((G.My, G.Mx), dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.StemError) as e:
        ctx.batch_device([], 0)
    assert e.value.code == _lib.ST_ERR_ARG
    with pytest.raises(_lib.StemError) as e:
        ctx.batch_device([(G, xd.data_ptr(), len(x), aa, im.data_ptr()), (G, 0, len(x), aa, im.data_ptr())], 0)
    assert e.value.code == _lib.ST_ERR_ARG and "job 1" in str(e.value)
    ctx.batch_device([(G, xd.data_ptr(), len(x), aa, im.data_ptr())], 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(im.cpu().numpy().T, ctx.image(G, x, aa))


@pytest.mark.parametrize("fp32", [False, True])
def test_capacity_retry_after_small_image(fp32):
    """The kept-atom arrays are sized by the previous call: a small image followed by a
    larger batch overflows them, and the batch is binned again into grown arrays."""
    flags = _lib.ST_FLAG_FP32 if fp32 else 0
    small = synth.small_cell(n=(6, 6, 4), seed=8, n_voids=0, with_screw=False)
    t, so, xs = _condition(small, sg=0.01)
    Gs, aas = t.image_geometry(len(xs))
    big = synth.small_cell(n=(30, 30, 12), seed=9, n_voids=2, radius=(4.0, 8.0), with_screw=True)
    tb, sob, xb = _condition(big, sg=0.01, density=True)
    Gb, aab = tb.image_geometry(len(xb), n_prec=2)
    fresh = imaging.Context(0)
    try:
        want_big = fresh.image(Gb, xb, aab, flags=flags | _lib.ST_FLAG_STATS)
        kept_big = fresh.stats().n_kept
    finally:
        fresh.close()
    c = imaging.Context(0)
    try:
        c.image(Gs, xs, aas, flags=flags | _lib.ST_FLAG_STATS)
        kept_small = c.stats().n_kept
        assert 2 * kept_big > kept_small + kept_small // 4 + 65536  # the batch cannot fit the first guess
        got = _batch(c, [(Gb, aab, xb), (Gs, aas, xs), (Gb, aab, xb)], flags | _lib.ST_FLAG_STATS)
        assert c.stats().n_kept == 2 * kept_big + kept_small
    finally:
        c.close()
    assert np.array_equal(got[0], want_big) and np.array_equal(got[2], want_big)
    Go, aao = O.geometry(sob, len(xb), nPrec=2, precAngle=0.005)
    want, _ = O.patch_image(Go, aao, xb, nthreads=8)
    assert np.abs(got[0] - want).max() <= (FP32_TOL if fp32 else FP64_TOL)


@pytest.mark.parametrize("fp32", [False, True])
def test_host_batch_equals_device_batch(ctx, fp32):
    """st_batch (host buffers, atoms shared by several jobs uploaded once, ldx = 14
    packed on the way) gives the images of st_batch_device."""
    flags = (_lib.ST_FLAG_FP32 if fp32 else 0) | _lib.ST_FLAG_AVERAGE
    specs, _ = _mixed_specs(fp32)
    G0, aa0, x0 = specs[0]
    x14 = np.zeros((len(x0), 14))
    x14[:, :3] = x0
    x14[:, 3:] = -3.0
    host_specs = [(G, x, aa) for G, aa, x in specs] + [(G0, x0, aa0), (G0, x14, aa0)]  # x0 twice: one upload
    got = ctx.batch(host_specs, flags)
    want = _batch(ctx, specs, flags)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    assert np.array_equal(got[-2], want[0]) and np.array_equal(got[-1], want[0])


def test_ring_variants_agree_and_autotuned():
    """The slab-ring variants (tile shape 8 x 4 / 4 x 8 / 16 x 2, slab
    capacity 96 / 128, CTAs per SM): every variant within the FP32 bar of the oracle;
    variants that differ only in slab capacity or occupancy compute the same image to the
    last bit.  With ST_TUNE_AUTO a context times them all on its first large pass, keeps
    the fastest, and its images are that variant's own."""
    cell = synth.make_cell(70, 70, 8, 11, n_voids=2, void_radius=(5.0, 8.0), with_screw=True)
    t, so, x = _condition(cell, sg=0.01, density=True)
    G, aa = t.image_geometry(len(x), n_prec=3)
    flags = _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE
    n_var = _lib.lib().st_tune_variants()
    assert n_var == 6
    imgs = []
    c = imaging.Context(0)
    try:
        for v in range(n_var):
            c.tune(v)
            imgs.append(c.image(G, x, aa, flags=flags))
            assert c.stats().ring_variant == v
            assert c.stats().ring_slab_atoms == (96 if v in (1, 3, 5) else 128)
        c.tune(_lib.ST_TUNE_AUTO)
        auto = c.image(G, x, aa, flags=flags)
        chosen = c.stats().ring_variant
        assert 0 <= chosen < n_var
        again = c.image(G, x, aa, flags=flags)
        assert c.stats().ring_variant == chosen
        with pytest.raises(_lib.StemError):
            c.tune(n_var)
    finally:
        c.close()
    for a_, b_ in ((0, 1), (2, 3), (4, 5)):
        assert np.array_equal(imgs[a_], imgs[b_])
    assert np.array_equal(auto, imgs[chosen]) and np.array_equal(again, imgs[chosen])
    Go, aao = O.geometry(so, len(x), nPrec=3, precAngle=0.005)
    want, _ = O.patch_image(Go, aao, x, nthreads=8)
    for im in imgs:
        d = im - want / 3
        assert np.abs(d).max() <= FP32_TOL
        assert np.sqrt((d ** 2).mean()) <= FP32_TOL / 5
    # the shapes sum each column's atoms in different orders: equal to FP32 rounding only
    assert max(np.abs(im - imgs[0]).max() for im in imgs) <= 2e-5


def _device_jobs(specs):
    """(G, aa, x) specs -> device buffers and (geom, x_ptr, n, aa, img_ptr) jobs."""
    dev, imgs, jobs = {}, [], []
    for G, aa, x in specs:
        if id(x) not in dev:
            dev[id(x)] = torch.from_numpy(np.ascontiguousarray(x)).to("cuda") if len(x) else \
                torch.zeros(3, dtype=torch.float64, device="cuda")
        im = torch.full((G.My, G.Mx), 7.0, dtype=torch.float64, device="cuda")
        imgs.append(im)
        jobs.append((G, dev[id(x)].data_ptr(), len(x), aa, im.data_ptr()))
    return dev, imgs, jobs


@pytest.mark.parametrize("fp32", [False, True])
def test_plan_replay_equals_batch(ctx, fp32):
    """A recorded plan replays the batch: its images equal st_batch_device's bit for bit,
    after the recording run and after every replay."""
    flags = (_lib.ST_FLAG_FP32 if fp32 else 0) | _lib.ST_FLAG_AVERAGE
    specs, _ = _mixed_specs(fp32)
    want = _batch(ctx, specs, flags)
    dev, imgs, jobs = _device_jobs(specs)
    torch.cuda.synchronize()
    plan = ctx.plan(jobs, flags)
    try:
        torch.cuda.synchronize()
        for a, b in zip(imgs, want):
            assert np.array_equal(a.cpu().numpy().T, b)
        for _ in range(3):
            for im in imgs:
                im.fill_(-1.0)
            torch.cuda.synchronize()
            plan.launch()
            plan.wait()
            for a, b in zip(imgs, want):
                assert np.array_equal(a.cpu().numpy().T, b)
    finally:
        plan.close()


def test_plan_follows_moving_atoms(ctx):
    """Positions rewritten in place between replays (a trajectory): each replay images
    the current positions, equal to a fresh call on them."""
    cell = synth.small_cell(n=(10, 10, 8), seed=5, n_voids=1, radius=(4.0, 6.0), with_screw=True)
    t, so, x = _condition(cell, sg=0.01, density=True)
    G, aa = t.image_geometry(len(x), n_prec=2)
    flags = _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE
    dev, imgs, jobs = _device_jobs([(G, aa, x)])
    d_x = dev[id(x)]
    torch.cuda.synchronize()
    plan = ctx.plan(jobs, flags)
    rng = np.random.default_rng(3)
    try:
        for frame in range(3):
            xf = x + rng.normal(0.0, 0.05, size=x.shape)
            d_x.copy_(torch.from_numpy(xf))
            torch.cuda.synchronize()
            plan.launch()
            plan.wait()
            assert np.array_equal(imgs[0].cpu().numpy().T, ctx.image(G, xf, aa, flags=flags))
    finally:
        plan.close()


def test_plan_recovers_from_slab_overflow(ctx):
    """A replay whose atoms overfill the ring kernel's slabs (even 256-atom ones: a ball at
    eight times the density) is recomputed on the eager path (general kernel) by
    st_plan_wait, then recorded again."""
    cell = synth.small_cell(n=(9, 11, 7), seed=6, n_voids=3, radius=(3.0, 5.0), with_screw=False)
    t, so, x = _condition(cell, sg=0.01)
    G, aa = t.image_geometry(len(x))
    flags = _lib.ST_FLAG_FP32
    dev, imgs, jobs = _device_jobs([(G, aa, x)])
    d_x = dev[id(x)]
    torch.cuda.synchronize()
    plan = ctx.plan(jobs, flags)
    try:
        assert plan.stats().column_kernel == 2
        # same atom count: the eighth of the atoms nearest the cell centre, eight times over
        q = len(x) // 8
        near = np.argsort(((x - x.mean(axis=0)) ** 2).sum(axis=1))[:q]
        dense = np.concatenate([x[near]] * 8 + [x[:len(x) - 8 * q]])
        d_x.copy_(torch.from_numpy(dense))
        torch.cuda.synchronize()
        plan.launch()
        plan.wait()
        assert plan.stats().column_kernel == 1
        want = ctx.image(G, dense, aa, flags=flags)
        assert ctx.stats().column_kernel == 1
        assert np.array_equal(imgs[0].cpu().numpy().T, want)
        # back to the original atoms: the re-recorded plan (general kernel) still images them
        d_x.copy_(torch.from_numpy(x))
        torch.cuda.synchronize()
        plan.launch()
        plan.wait()
        Go, aao = O.geometry(so, len(x))
        ref, _ = O.patch_image(Go, aao, x, nthreads=8)
        assert np.abs(imgs[0].cpu().numpy().T - ref).max() <= FP32_TOL
    finally:
        plan.close()


def test_batch_stats_report_the_variant():
    """A batch's statistics (its binning groups merged) name the slab-ring variant that ran
    and its staging capacity, as a single image's do."""
    specs, _ = _mixed_specs(True)
    c = imaging.Context(0)
    try:
        c.tune(3)
        _batch(c, specs, _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE)
        st = c.stats()
        assert st.column_kernel == 2
        assert st.ring_variant == 3
        assert st.ring_slab_atoms in (96, 192, 256)  # the variant's tier, or a larger one after an overflow
    finally:
        c.close()


def test_autotuner_keys_on_image_shape():
    """With ST_TUNE_AUTO the first large image of each shape in a context times the variants
    (more kernel launches than a plain call); the next image of that shape reuses the choice."""
    cell = synth.make_cell(100, 100, 8, 13, n_voids=2, void_radius=(5.0, 8.0), with_screw=True)
    jobs = []
    for M in ((4, 4), (5, 5)):
        t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.01, M=M)
        G, aa = t.image_geometry(len(x))
        assert ((G.ix1 - G.ix0 + 7) // 8) * ((G.iy1 - G.iy0 + 3) // 4) >= 4096  # large enough to tune
        jobs.append((G, x, aa))
    assert (jobs[0][0].Mx, jobs[0][0].My) != (jobs[1][0].Mx, jobs[1][0].My)
    c = imaging.Context(0)
    try:
        launches, variants = [], []
        for G, x, aa in jobs + jobs:
            c.image(G, x, aa, flags=_lib.ST_FLAG_FP32)
            launches.append(c.stats().n_launches)
            variants.append(c.stats().ring_variant)
    finally:
        c.close()
    assert launches[0] > launches[2] and launches[1] > launches[3]
    assert variants[2] == variants[0] and variants[3] == variants[1]
