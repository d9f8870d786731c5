"""The -ng tilt search (setSupercellTilt1a): the oracle pinned to the reference's own
golden run, and the host steps of the product (reflections, extinction table, golden
section, quaternions) against the oracle.  CPU only; the GPU scores are in
test_gpu_tilt.py."""
import ctypes
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import imaging as I
from simulated_tem_gb300 import _lib
from tests import golden_data

XI = os.path.join(golden_data.GOLDEN, "w_xi_V200_T300.dat")
HUGE1 = float(np.finfo(np.float32).max)


@pytest.fixture(scope="module")
def w_loop_ng():
    """The testD2BI run itself: -a0 3.1652 -lattice bcc -k 0,0,1 -g 2,0,0 -xifile ... -ng 1."""
    g = golden_data.w_loop()
    args = O.make_args(g["a_super"], 3.1652, (0, 0, 1), (2, 0, 0), V=200.0, M=(4, 4), ng=1.0, xifile=XI, dark=True)
    state, x, aperpx = O.setup(args, g["pos"])
    return g, state, x, aperpx


def _cm(a):
    return np.array(list(a)).reshape(3, 3).T


def test_oracle_tilt_search_reproduces_golden_header(w_loop_ng):
    """Data/test/*.dat header: rotation matmul(R, U) (6 decimals), s_g (5), image box (3),
    pixel scale (5), xi values (5) and the 94 x 94 x 95 voxel grid."""
    g, t, _, aperpx = w_loop_ng
    h = g["header"]
    RU = _cm(t.R) @ _cm(t.U)
    assert np.abs(RU - g["RU"]).max() <= 5.0e-7
    assert "%.5f" % t.sg == "%.5f" % h["s_g (1/A)"][0]
    assert ["%.3f" % v for v in t.voxelSupercellDimensions] == ["%.3f" % v for v in h["img space (A)"]]
    assert "%.5f" % aperpx == "%.5f" % h["scale (A/px)"][0]
    assert ("%.5f" % t.xi0, "%.5f" % t.xig) == ("%.5f" % h["xi (A)"][0], "%.5f" % h["xi (A)"][1])
    assert (t.gksuper.Nx, t.gksuper.Ny, t.gksuper.Nz) == (94, 94, 95)


def test_oracle_ng_image_matches_golden_dat_to_its_rounding(w_loop_ng):
    """With the tilt found by the search the restated image equals the shipped .dat to the
    7-decimal rounding of the file (the header-rotation route is only good to 1e-4)."""
    g, t, x, _ = w_loop_ng
    img, _ = O.compute_d2bi_img(t, x, nthreads=4)
    assert np.abs(img - g["img"]).max() <= 5.0e-8 + 1e-12


def test_oracle_search_statistics():
    """The search the golden run made: 4,000 candidate directions, 2,123 bcc reflections
    within RHO_MAX = 10, every xi found, the first THETA_MAX attempt."""
    v = O.lib().oc_velocity(O._d(200000.0))
    U, R, info, scores, khat = O.find_best_rotation(v, (0, 0, 1), 3.1652 * np.eye(3), "bcc", (2, 0, 0), XI,
                                                    74.88124812040851)
    assert (info.nk, info.nn, info.attempt, info.xi_ok) == (4000, 2123, 1, 1)
    assert info.ii_best == int(np.argmin(scores)) + 1
    assert np.allclose(np.linalg.norm(khat, axis=1), 1.0, atol=1e-14)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-14) and R[2, 2] > 0


@pytest.mark.parametrize("lattice,rho", [("sc", 4.0), ("bcc", 10.0), ("fcc", 7.5), ("hcp", 6.3), ("bcc", 0.0)])
def test_permitted_reflections_match_oracle(lattice, rho):
    h = I.permitted_reflections(lattice, rho)
    assert np.array_equal(h, O.permitted_reflections(lattice, rho))
    if lattice == "bcc":
        assert np.all((h.sum(axis=1) % 2) == 0)
    assert [0, 0, 0] in h.tolist()


def test_extinction_table_matches_oracle_and_symmetry():
    h = I.permitted_reflections("bcc", 10.0)
    xi, st = I.read_extinction_distances(XI, h)
    xo, so = O.read_extinction_distances(XI, h)
    assert st == so == 1 and np.array_equal(xi, xo)
    # the table lists standard forms only: [-2,0,0], [0,0,2] and [0,2,0] read [2,0,0]'s xi
    x3, _ = I.read_extinction_distances(XI, [[-2, 0, 0], [0, 0, 2], [0, 2, 0], [2, 0, 0]])
    assert len(set(x3.tolist())) == 1 and x3[0] == 308.24708823
    assert I.read_extinction_distances(XI, [[0, 0, 0]])[0][0] == 113.88928751


def test_extinction_table_edge_cases(tmp_path):
    p = str(tmp_path / "t.dat")
    # missing file: status -1, every xi huge(1.0)
    xi, st = I.read_extinction_distances(p, [[1, 1, 0]])
    assert st == -1 and xi[0] == HUGE1
    # header only: nothing found
    with open(p, "w") as f:
        f.write("# t\n element g T V ReU ImU xi\n")
    xi, st = I.read_extinction_distances(p, [[1, 1, 0]])
    assert (st, xi[0]) == (0, HUGE1)
    assert O.read_extinction_distances(p, [[1, 1, 0]])[1] == 0
    # a record split over two lines, a Fortran D exponent, commas; then a malformed record ends the read
    with open(p, "w") as f:
        f.write("# t\n element g T V ReU ImU xi\n")
        f.write("Fe 1 1 0 300.0\n 200000.0, 1.0 0.5 3.3D2\n")
        f.write("Fe 2 0 0 300.0 200000.0 1.0 0.5 1.5e2\n")
        f.write("Fe 2 1 1 300.0 x 1.0 0.5 9.0\n")
        f.write("Fe 2 2 0 300.0 200000.0 1.0 0.5 7.0\n")
    want = [[0, 1, -1], [0, 0, 2], [-1, 2, 1], [2, 2, 0]]
    xi, st = I.read_extinction_distances(p, want)
    xo, so = O.read_extinction_distances(p, want)
    assert st == so == 0
    assert np.array_equal(xi, xo)
    assert xi.tolist() == [330.0, 150.0, HUGE1, HUGE1]


def test_hexagonal_standard_forms(tmp_path):
    p = str(tmp_path / "h.dat")
    with open(p, "w") as f:
        f.write("# t\n element g T V ReU ImU xi\n")
        f.write("Ti 1 0 0 300 200000 1 1 111.0\n")
        f.write("Ti 1 -1 2 300 200000 1 1 222.0\n")
        f.write("Ti 2 1 1 300 200000 1 1 333.0\n")
    want = [[0, 1, 0], [-1, 0, 0], [-1, 1, 2], [1, -1, -2], [1, 2, 1], [-2, -1, 1]]
    xi, st = I.read_extinction_distances(p, want, lattice="hcp")
    xo, so = O.read_extinction_distances(p, want, symm=2)
    assert st == so and np.array_equal(xi, xo)
    assert xi.tolist() == [111.0, 111.0, 222.0, 222.0, 333.0, 333.0]


def _rot(axis, angle):
    axis = np.asarray(axis, dtype=np.float64) / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


@pytest.mark.parametrize("axis,angle", [((1, 0, 0), 0.01), ((0.3, -0.2, 0.9), 0.7), ((0, 1, 0), 2.9),
                                        ((1, 1, 1), 0.0)])
def test_quaternion_round_trip_matches_oracle(axis, angle):
    """RotMatToQuaternion (DSYEV's dominant eigenvector) and quaternionToRotMat."""
    R = _rot(axis, angle)
    L = _lib.lib()
    q = (ctypes.c_double * 4)()
    assert L.st_rotmat_to_quaternion(I._cm(R), q) == 0
    Ro, qo = O.quaternion_round_trip(R)
    assert list(q) == list(qo)  # the same restatement, bit for bit
    assert q[0] >= 0 and abs(q[0] - np.cos(angle / 2)) < 1e-14
    back = (ctypes.c_double * 9)()
    assert L.st_quaternion_to_rotmat(q, back) == 0
    assert np.array_equal(I._from_cm(back), Ro)
    assert np.abs(I._from_cm(back) - R).max() < 1e-14


@pytest.mark.parametrize("x", [0.0, 0.25, 0.5, 1.0])
def test_slerp_matches_oracle(x):
    L = _lib.lib()
    q1 = np.array([np.cos(0.1), np.sin(0.1), 0.0, 0.0])
    q2 = np.array([np.cos(0.3), 0.0, np.sin(0.3) * 0.6, np.sin(0.3) * 0.8])
    out = (ctypes.c_double * 4)()
    assert L.st_slerp(I._ptr(q1), I._ptr(q2), x, out) == 0
    ref = (ctypes.c_double * 4)()
    O.lib().oc_slerp(O._dptr(q1), O._dptr(q2), O._d(x), ref)
    assert list(out) == list(ref)
    assert abs(np.linalg.norm(list(out)) - 1) < 1e-15
    same = (ctypes.c_double * 4)()
    assert L.st_slerp(I._ptr(q1), I._ptr(q1), x, same) == 0
    assert np.abs(np.array(list(same)) - q1).max() < 1e-15


@pytest.mark.parametrize("foil,xig", [(74.88124812040851, 207.5), (150.0, 300.0), (40.0, 120.0)])
def test_tilt_to_dark_field_matches_oracle(foil, xig):
    """tiltToDarkField: the golden-section search of |phi_g(L')|^2 over a tilt about y."""
    a_cell = 3.1652 * np.eye(3)
    v = O.lib().oc_velocity(O._d(200000.0))
    R0 = _rot((0.2, 1.0, 0.1), 0.02)
    U = np.eye(3)
    R = np.array(R0)
    Rc = I._cm(R)
    th = ctypes.c_double()
    h = (ctypes.c_int32 * 3)(2, 0, 0)
    assert _lib.lib().st_tilt_to_dark_field(v, I._cm(a_cell), h, 103.9, xig, foil, 5.0, I._cm(U), Rc,
                                             ctypes.byref(th)) == 0
    Ro = O._mat(R0)
    tho = O._d()
    assert O.lib().oc_tilt_to_dark_field(O._d(v), O._mat(a_cell), (ctypes.c_int * 3)(2, 0, 0), O._d(103.9),
                                         O._d(xig), O._d(foil), O._d(5.0), O._mat(U), Ro, ctypes.byref(tho)) == 0
    assert list(Rc) == list(Ro) and th.value == tho.value
    # the bracket starts at +-THETA_MAX / 100 and may grow for up to ten steps while unbounded
    assert abs(th.value) < 0.1


def test_condition_api_requires_context_for_ng():
    g = golden_data.w_loop()
    with pytest.raises(_lib.StemError):
        I.d2bi_condition(g["a_super"], 3.1652, (0, 0, 1), (2, 0, 0), g["pos"], ng=1.0, xifile=XI)


def test_quaternion_kat():
    """test/testLib_Quaternions.f90: RotMatToQuaternion of its matrix, '(4f16.8)'."""
    import json
    with open(os.path.join(golden_data.GOLDEN, "quaternion_kat.json")) as f:
        k = json.load(f)
    R = np.array(k["R1_column_major"]).reshape(3, 3).T
    _, qo = O.quaternion_round_trip(R)
    assert ["%.8f" % v for v in qo] == k["q_wxyz"]
    q = (ctypes.c_double * 4)()
    assert _lib.lib().st_rotmat_to_quaternion(I._cm(R), q) == 0
    assert ["%.8f" % v for v in q] == k["q_wxyz"]


def test_golden_section_kat():
    """test/testLib_GoldenSection.f90: from each of its brackets the search ends at a local
    minimum of the test's function (all seven, the test's pass count)."""
    import json
    import math
    with open(os.path.join(golden_data.GOLDEN, "golden_section_kat.json")) as f:
        k = json.load(f)

    def func(x):  # the test program's function
        if x < 0:
            return HUGE1
        return 1.0 + x * (1.0 + x * (-0.1 + x * 0.2)) * math.sin(3 * x) + math.cos(x) * math.sqrt(x)

    cb = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double, ctypes.c_void_p)(lambda x, _: func(x))
    passes = 0
    for x1, x3 in k["brackets"]:
        xt, yt = ctypes.c_double(), ctypes.c_double()
        steps = O.lib().oc_golden_minimise(O._d(x1), O._d(x3), cb, None, ctypes.byref(xt), ctypes.byref(yt))
        assert steps > 0
        if min(func(xt.value + 0.001), func(xt.value - 0.001)) > func(xt.value):
            passes += 1
    assert passes == k["pass_count"]
