"""The -ng tilt search with its scores on the GPU: the scores against the oracle's, the
search's choice and the whole set-up (rotation, deviation parameter, voxel geometry) bit
for bit equal to the oracle's, and the testD2BI run itself through the GPU imaging path
against the reference's shipped image."""
import ctypes
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import _lib, imaging, synth
from tests import golden_data
from tests.test_host_geometry import assert_geom_equal

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

XI = os.path.join(golden_data.GOLDEN, "w_xi_V200_T300.dat")
FOIL = 74.88124812040851  # the W loop's atom depth after rotation to [001] / [200]


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def w_loop():
    return golden_data.w_loop()


def _velocity():
    return O.lib().oc_velocity(O._d(200000.0))


def test_scores_match_oracle(ctx):
    """Every candidate's score: the sine and cosine of the two phases are CUDA's and the
    lanes' sum order differs, nothing else; the difference stays within the bound the
    host uses to resolve near-ties."""
    v = _velocity()
    a_cell = 3.1652 * np.eye(3)
    _, _, info, scores, khat = O.find_best_rotation(v, (0, 0, 1), a_cell, "bcc", (2, 0, 0), XI, FOIL)
    g, xi = O.tilt_reflections("bcc", a_cell, (2, 0, 0), XI)
    assert len(g) == info.nn == 2123
    gpu = imaging.tilt_scores(ctx, v, khat, g, xi, FOIL)
    nn = len(g)
    bound = 8.0 * (nn * 4.0e-15 + nn * 2.3e-16 * np.abs(gpu))
    assert np.all(np.abs(gpu - scores) <= bound)
    assert np.abs(gpu - scores).max() < 1e-11
    assert int(np.argmin(gpu)) == info.ii_best - 1


@pytest.mark.parametrize("z0,hkl,foil", [((0, 0, 1), (2, 0, 0), FOIL), ((0, 0, 1), (1, 1, 0), 400.0),
                                         ((1, 1, 1), (1, -1, 0), 60.0), ((0, 0, 1), (4, 0, 0), 1200.0)])
def test_screen_bounds_hold(ctx, z0, hkl, foil):
    """The FP32 screen's bound covers its distance from the FP64 score for every direction,
    and the bound is tight enough to leave few directions to the FP64 pass."""
    v = _velocity()
    a_cell = 3.1652 * np.eye(3)
    _, _, info, scores, khat = O.find_best_rotation(v, z0, a_cell, "bcc", hkl, XI, foil)
    g, xi = O.tilt_reflections("bcc", a_cell, hkl, XI)
    s32, b32 = imaging.tilt_screen(ctx, v, khat, g, xi, foil)
    assert np.all(np.abs(s32 - scores) <= b32)
    lim = np.min(s32 + b32)
    assert int(np.sum(s32 - b32 <= lim)) <= len(khat) // 4


def test_best_rotation_equals_oracle(ctx):
    v = _velocity()
    a_cell = 3.1652 * np.eye(3)
    for z0, hkl, foil in (((0, 0, 1), (2, 0, 0), FOIL), ((0, 0, 1), (1, 1, 0), 120.0), ((1, 1, 1), (1, -1, 0), 60.0),
                          ((0, 0, 1), (4, 0, 0), 200.0)):
        U, R, info = imaging.find_best_rotation(ctx, v, z0, a_cell, "bcc", hkl, XI, foil)
        Uo, Ro, io, _, _ = O.find_best_rotation(v, z0, a_cell, "bcc", hkl, XI, foil)
        assert np.array_equal(U, Uo) and np.array_equal(R, Ro), (z0, hkl)
        assert (info["nk"], info["nn"], info["ii_best"], info["attempt"]) == (io.nk, io.nn, io.ii_best, io.attempt)
        assert info["ss_best"] == io.ss_best
        assert 1 <= info["n_recheck"] <= 64
        assert 1 <= info["n_fp64"] < info["nk"] // 4
        assert info["scan_ms"] > 0 and 0 < info["screen_ms"] <= info["scan_ms"]


def _product_ng(ctx, cell, a0, k, g, ng, **kw):
    return imaging.d2bi_condition(cell.a_super, a0, k, g, cell.pos, ng=ng, xifile=XI, ctx=ctx, **kw)


def _oracle_ng(cell, a0, k, g, ng, **kw):
    args = O.make_args(cell.a_super, a0, k, g, ng=ng, xifile=XI, **kw)
    return O.setup(args, cell.pos)


def test_w_loop_ng_setup_equals_oracle_and_golden(ctx, w_loop):
    cell = synth.Cell(w_loop["a_super"], w_loop["pos"])
    t, xw, ap = _product_ng(ctx, cell, 3.1652, (0, 0, 1), (2, 0, 0), 1.0)
    so, xo, apo = _oracle_ng(cell, 3.1652, (0, 0, 1), (2, 0, 0), 1.0)
    assert np.array_equal(xw, xo) and ap == apo
    U, R = t.get_rotation()
    assert np.array_equal(U, np.array(list(so.U)).reshape(3, 3).T)
    assert np.array_equal(R, np.array(list(so.R)).reshape(3, 3).T)
    assert t.get_deviation_parameter() == so.sg
    Gp, aap = t.image_geometry(len(xw))
    Go, aao = O.geometry(so, len(xo))
    assert_geom_equal(Gp, aap, Go, aao)
    assert np.abs(R @ U - w_loop["RU"]).max() <= 5e-7  # the header's 6 decimals
    assert t.tilt["nk"] == 4000 and t.tilt["nn"] == 2123


def test_w_loop_ng_image_matches_shipped_dat(ctx, w_loop):
    """The testD2BI run end to end on the GPU: the FP64 image equals the shipped .dat to its
    7-decimal rounding; the FP32 path stays within 1e-4."""
    cell = synth.Cell(w_loop["a_super"], w_loop["pos"])
    t, xw, _ = _product_ng(ctx, cell, 3.1652, (0, 0, 1), (2, 0, 0), 1.0)
    img = t.compute_d2bi_img(ctx, xw, n_prec=1)
    assert img.shape == (94, 94)
    assert np.abs(img - w_loop["img"]).max() <= 5.0e-8 + 1e-12
    img32 = t.compute_d2bi_img(ctx, xw, n_prec=1, flags=_lib.ST_FLAG_FP32)
    assert np.abs(img32 - w_loop["img"]).max() <= 1e-4


@pytest.mark.parametrize("ng", [1.5, 2.0])
def test_fractional_and_higher_ng_equal_oracle(ctx, ng):
    """(g, ng) with ng = 2 (hkl = 400) and ng = 1.5: two searches and a slerp."""
    cell = synth.small_cell((12, 12, 10), seed=7)
    t, xw, _ = _product_ng(ctx, cell, synth.A0_FE, (0, 0, 1), (1, 1, 0), ng)
    so, xo, _ = _oracle_ng(cell, synth.A0_FE, (0, 0, 1), (1, 1, 0), ng)
    U, R = t.get_rotation()
    assert np.array_equal(R, np.array(list(so.R)).reshape(3, 3).T)
    assert np.array_equal(U, np.array(list(so.U)).reshape(3, 3).T)
    assert t.get_deviation_parameter() == so.sg
    Gp, aap = t.image_geometry(len(xw))
    Go, aao = O.geometry(so, len(xo))
    assert_geom_equal(Gp, aap, Go, aao)


def test_surface_foil_thickness_equals_oracle(ctx):
    """-surf: the foil thickness from the atoms (27 replicas, columns of about 3 a0) on the
    GPU, for a slab with vacuum above and below."""
    cell = synth.small_cell((14, 14, 10), seed=5)
    a_super = np.array(cell.a_super, dtype=np.float64)
    a_super[2, 2] *= 1.6  # vacuum: the atoms fill 10 of 16 cells in z
    slab = synth.Cell(a_super, cell.pos + np.array([0.0, 0.0, 0.3 * a_super[2, 2] / 1.6]))
    t, xw, _ = _product_ng(ctx, slab, synth.A0_FE, (0, 0, 1), (1, 1, 0), 1.0, surf=True, d=(40.0, 40.0, 46.0))
    so, xo, _ = _oracle_ng(slab, synth.A0_FE, (0, 0, 1), (1, 1, 0), 1.0, surf=True, d=(40.0, 40.0, 46.0))
    U, R = t.get_rotation()
    assert np.array_equal(R, np.array(list(so.R)).reshape(3, 3).T)
    assert t.get_deviation_parameter() == so.sg
    info = t.tilt
    assert 0 < info["foil"] < 46.0
    # the atoms span about 10 cells of 2.87 A less a column's roughness
    assert abs(info["foil"] - 10 * synth.A0_FE) < 3 * synth.A0_FE
    Gp, aap = t.image_geometry(len(xw))
    Go, aao = O.geometry(so, len(xo))
    assert_geom_equal(Gp, aap, Go, aao)


def test_tilt_search_argument_errors(ctx):
    v = _velocity()
    with pytest.raises(_lib.StemError):
        imaging.find_best_rotation(ctx, v, (0, 0, 1), 3.1652 * np.eye(3), "bcc", (2, 0, 0), XI, 74.0, theta_max=0.0)
    with pytest.raises(_lib.StemError):
        imaging.tilt_scores(ctx, v, np.zeros((0, 3)), np.zeros((4, 3)), np.ones(4), 10.0)
    # a missing table is not an error in the reference: every xi_g stays huge(1.0)
    U, R, info = imaging.find_best_rotation(ctx, v, (0, 0, 1), 3.1652 * np.eye(3), "bcc", (2, 0, 0),
                                            "/nonexistent/xi.dat", 74.0)
    Uo, Ro, io, _, _ = O.find_best_rotation(v, (0, 0, 1), 3.1652 * np.eye(3), "bcc", (2, 0, 0),
                                            "/nonexistent/xi.dat", 74.0)
    assert info["xi_status"] == -1 and np.array_equal(R, Ro)
