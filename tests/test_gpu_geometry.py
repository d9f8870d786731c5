"""The passes over the atoms of d2bi's set-up on the GPU (the periodic wrap and the
rotated atom extents) give the host mirror's bits, so a sweep set up on the device has the
same geometry, image for image, as one set up condition by condition on the host."""
import ctypes

import numpy as np
import pytest

from simulated_tem_gb300 import _lib, imaging, synth

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def cell():
    return synth.make_cell(30, 24, 20, synth.BASE_SEED + 11, n_voids=4, void_radius=(4.0, 8.0), with_screw=True)


def test_wrap_matches_host(ctx, cell):
    a0 = synth.A0_FE
    xw, a_vox, n = imaging.wrap_pbc(cell.a_super, (4, 4), a0, cell.pos)
    d = torch.from_numpy(np.ascontiguousarray(cell.pos)).cuda()
    ctx._check(imaging.lib().st_wrap_pbc_device(ctx.handle, imaging._cm(a_vox), n[0], n[1], n[2],
                                                ctypes.c_void_p(d.data_ptr()), 3, len(cell.pos), None))
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), xw)


def test_extents_match_host(ctx, cell):
    a0 = synth.A0_FE
    xw, _, _ = imaging.wrap_pbc(cell.a_super, (4, 4), a0, cell.pos)
    conds = [((0, 0, 1), (1, 1, 0)), ((0, 0, 1), (2, 0, 0)), ((0, 0, 1), (2, 1, 1)), ((1, 1, 1), (1, -1, 0)),
             ((0, 1, 1), (2, 0, 0))]
    nc = len(conds)
    ks = (ctypes.c_double * (3 * nc))(*[float(v) for k, _ in conds for v in k])
    gs = (ctypes.c_double * (3 * nc))(*[float(v) for _, g in conds for v in g])
    dd = (ctypes.c_double * (3 * nc))()
    d = torch.from_numpy(xw).cuda()
    ctx._check(imaging.lib().st_atom_extents_device(ctx.handle, nc, ks, gs, imaging._cm(a0 * np.eye(3)),
                                                    ctypes.c_void_p(d.data_ptr()), 3, len(xw), dd))
    for c, (k, g) in enumerate(conds):
        assert list(dd[3 * c:3 * c + 3]) == imaging.atom_extents(k, g, a0 * np.eye(3), xw)


def test_sweep_set_up_on_device_equals_host(ctx, cell):
    gs = [(1, 1, 0), (2, 0, 0), (2, 1, 1)]
    d_x, specs, _ = imaging.d2bi_sweep(ctx, cell.a_super, synth.A0_FE, (0, 0, 1), gs, cell.pos, n_tomo=7,
                                       tomo_angle=20.0, prec_angle=0.005, n_prec=4, sg=0.01, xi0=103.9, xig=207.5)
    i = 0
    for g in gs:
        for step in range(7):
            t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), g, cell.pos, sg=0.01, xi0=103.9,
                                             xig=207.5, n_tomo=7, tomo_angle=20.0, tomo_step=step)
            G, aa = t.image_geometry(len(x), prec_angle=0.005, n_prec=4)
            Gd, aad = specs[i]
            assert bytes(G) == bytes(Gd) and np.array_equal(aa, aad), (g, step)
            i += 1
    assert np.array_equal(d_x.cpu().numpy(), x)


def _oracle_sweep_geometry(cell, g, n_tomo, step, n_prec):
    from oracle import stem_oracle as O
    args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), g, sg=0.01, xi0=103.9, xig=207.5, nTomo=n_tomo,
                       tomoAngle=20.0)
    so, xo, _ = O.setup(args, cell.pos, nn=step)
    Go, aao = O.geometry(so, len(xo), nPrec=n_prec, precAngle=0.005)
    return xo, Go, aao


@pytest.mark.parametrize("which", ["small", "1p2m"])
def test_sweep_geometry_matches_oracle(ctx, cell, which):
    """d2bi_sweep (the wrap and the extents of every g on the GPU, the scalar set-up per tilt
    on the host) against the oracle's own set-up of each condition, tilt by tilt and g by g:
    the wrapped atoms, every field of the geometry the kernels receive, and the precession
    coefficients, all to the last bit.  The small cell: every one of 3 g x 9 tilts; the
    1.2M-atom cell of the benchmark's sweep (41 tilts): the first, middle and last tilt of
    each g."""
    from tests.test_host_geometry import assert_geom_equal
    gs = ((1, 1, 0), (2, 0, 0), (2, 1, 1))
    if which == "small":
        c, n_tomo, steps = cell, 9, range(9)
    else:
        c, n_tomo, steps = synth.screw_cell_1p2m(), 41, (0, 20, 40)
    d_x, specs, _ = imaging.d2bi_sweep(ctx, c.a_super, synth.A0_FE, (0, 0, 1), gs, c.pos, n_tomo=n_tomo,
                                       tomo_angle=20.0, prec_angle=0.005, n_prec=16, sg=0.01, xi0=103.9,
                                       xig=207.5)
    x_dev = d_x.cpu().numpy()
    for gi, g in enumerate(gs):
        for step in steps:
            xo, Go, aao = _oracle_sweep_geometry(c, g, n_tomo, step, 16)
            assert np.array_equal(xo, x_dev)
            G, aa = specs[gi * n_tomo + step]
            assert_geom_equal(G, aa, Go, aao)
