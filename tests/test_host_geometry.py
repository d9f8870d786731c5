"""The library's host mirror of the Fortran set-up (include/stem_host.h) against
the oracle's restatement: both restate the same reference routines, so the
geometry handed to the kernels must agree to the last bit.  CPU only."""
import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import imaging, synth
from tests import golden_data


def oracle_run(cell, a0, k, g, **kw):
    args = O.make_args(cell.a_super, a0, k, g, **{kk: v for kk, v in kw.items() if kk not in ("nn",)})
    return O.setup(args, cell.pos, nn=kw.get("nn", 0))


def product_run(cell, a0, k, g, **kw):
    m = dict(V=kw.get("V", 200.0), M=kw.get("M", (4, 4)), sg=kw.get("sg"), R=kw.get("R"), U=kw.get("U"),
             d=kw.get("d"), xi0=kw.get("xi0", 103.889565), xig=kw.get("xig", 207.533203),
             density=kw.get("density", False), n_tomo=kw.get("nTomo", 1), tomo_angle=kw.get("tomoAngle", 20.0),
             tomo_step=kw.get("nn", 0))
    return imaging.d2bi_condition(cell.a_super, a0, k, g, cell.pos, **m)


def assert_geom_equal(Gp, aap, Go, aao):
    for f in ("Mx", "My", "Mz", "ix0", "ix1", "iy0", "iy1", "Ex", "Ey", "Ez", "nMax0", "nuvw", "useDensity"):
        assert getattr(Gp, f) == getattr(Go, f), f
    for f in ("RU", "delta", "lc_delta", "a_col", "ia_col", "a_vox", "g"):
        assert list(getattr(Gp, f)) == list(getattr(Go, f)), f
    assert list(Gp.Ruvw)[:3 * Gp.nuvw] == list(Go.Ruvw)[:3 * Go.nuvw]
    for f in ("sigma", "deltaz", "b0", "bg"):
        assert getattr(Gp, f) == getattr(Go, f), f
    assert np.array_equal(aap, aao)


CASES = {
    "sg0": dict(sg=0.0),
    "sg0.01-density": dict(sg=0.01, density=True),
    "sg-neg": dict(sg=-0.015),
    "default": dict(),
    "tomo": dict(sg=0.01, nTomo=5, tomoAngle=20.0, nn=1),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("nprec", [1, 4])
def test_host_geometry_matches_oracle(case, nprec):
    cell = synth.small_cell((10, 10, 8), seed=11)
    kw = CASES[case]
    t, xw, ap = product_run(cell, synth.A0_FE, (0, 0, 1), (1, 1, 0), **kw)
    so, xo, apo = oracle_run(cell, synth.A0_FE, (0, 0, 1), (1, 1, 0), **kw)
    assert np.array_equal(xw, xo)
    assert ap == apo
    assert t.get_deviation_parameter() == so.sg
    for nprocs in (1, 2, 4):
        for jj in range(nprocs):
            Gp, aap = t.image_geometry(len(xw), prec_angle=0.005, n_prec=nprec, nprocs=nprocs, jj=jj)
            Go, aao = O.geometry(so, len(xo), nPrec=nprec, precAngle=0.005, nProcs=nprocs, jj=jj)
            assert_geom_equal(Gp, aap, Go, aao)


def test_host_geometry_w_loop_matches_oracle():
    g = golden_data.w_loop()
    cell = synth.Cell(g["a_super"], g["pos"])
    kw = dict(R=g["RU"], U=np.eye(3), d=g["d"], xi0=g["xi0"], xig=g["xig"])
    t, xw, _ = product_run(cell, 3.1652, (0, 0, 1), (2, 0, 0), **kw)
    so, xo, _ = oracle_run(cell, 3.1652, (0, 0, 1), (2, 0, 0), **kw)
    assert np.array_equal(xw, xo)
    Gp, aap = t.image_geometry(len(xw))
    Go, aao = O.geometry(so, len(xo))
    assert_geom_equal(Gp, aap, Go, aao)
    assert (Gp.Mx, Gp.My, Gp.Mz) == (94, 94, 95)


def test_rotation_and_image_parameters():
    cell = synth.small_cell((10, 10, 8), seed=3)
    t, _, _ = product_run(cell, synth.A0_FE, (0, 0, 1), (1, 1, 0), sg=0.01)
    U, R = t.get_rotation()
    assert np.allclose(U @ U.T, np.eye(3), atol=1e-12)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-12)
    assert abs(t.get_deviation_parameter() - 0.01) < 2e-4
    ap, xmax, modg, Mx, My, Mz = t.find_image_parameters()
    assert abs(modg - 2 * np.pi * np.sqrt(2) / synth.A0_FE) < 1e-12
    assert Mx >= 4 and My >= 4 and Mz >= 4 and ap > 0
