"""Pins the oracle (the CPU restatement of the reference) to the reference's
own golden vectors.  These run on CPU only."""
import numpy as np
import pytest

from oracle import stem_oracle as O
from tests import golden_data


@pytest.fixture(scope="module")
def w_loop_run():
    g = golden_data.w_loop()
    # The shipped image was made with -ng 1; its header records the resulting
    # matmul(R, U) and image box, which -R/-U/-d reproduce without the tilt search.
    args = O.make_args(g["a_super"], 3.1652, (0, 0, 1), (2, 0, 0), V=200.0, M=(4, 4), R=g["RU"], U=np.eye(3),
                       d=g["d"], xi0=g["xi0"], xig=g["xig"], dark=True)
    state, x, aperpx = O.setup(args, g["pos"])
    img, st = O.compute_d2bi_img(state, x, nthreads=4)
    return g, state, img, st, aperpx


def test_w_loop_image_matches_shipped_dat(w_loop_run):
    """Data/test/*.dat: the full 94x94 dark-field image (7 decimals)."""
    g, state, img, st, _ = w_loop_run
    assert (state.gksuper.Nx, state.gksuper.Ny, state.gksuper.Nz) == (94, 94, 95)
    d = img - g["img"]
    # the header rotation is rounded to 6 decimals: the residual is that rounding
    assert np.abs(d).max() < 2e-4
    assert np.sqrt((d ** 2).mean()) < 2e-5
    assert abs(state.sg - g["header"]["s_g (1/A)"][0]) < 1e-5


def test_w_loop_ctest_minmaxavg(w_loop_run):
    """test/testD2BI.sh:18-38: min/max/avg with the ctest's own acceptance window."""
    _, _, img, _, _ = w_loop_run
    acc = 0.0039
    for v, t in ((img.min(), 0.000028), (img.max(), 0.230127), (img.mean(), 0.081501)):
        assert int(abs((v - t) / acc + 0.5)) == 0


def test_w_loop_png_blur_and_levels(w_loop_run):
    """Data/test/*.png: blur(t = png_blur / aperpx) and the 16-bit normalisation."""
    g, _, img, _, aperpx = w_loop_run
    hx = g["d"]
    ap = np.sqrt(hx[0] * hx[1] / (94 * 94))
    lv = O.png_levels(O.gaussian_blur(g["img"], 2.5 / ap)).astype(int)
    assert np.abs(lv - g["png"].astype(int)).max() <= 1
    lv2 = O.png_levels(O.gaussian_blur(img, 2.5 / aperpx)).astype(int)
    assert np.abs(lv2 - g["png"].astype(int)).max() <= 8


def test_linkcell_neighbour_list_kat():
    """test/testLib_LinkCell3D.f90: the stored neighbours of atom 100."""
    k = golden_data.linkcell_kat()
    pts = np.array(k["points"])
    ids, dx, r2, max_count = O.neighbour_list(np.eye(3), k["cells"], 6, pts, pts[99], k["cutoff"])
    assert list(ids) == [n["id"] for n in k["neighbours"]]
    assert np.abs(dx - np.array([n["dx"] for n in k["neighbours"]])).max() < 1e-8
    assert np.abs(np.sqrt(r2) - np.array([n["absdx"] for n in k["neighbours"]])).max() < 1e-8
    assert max_count == k["max_count"]


def test_electron_wavelength_kat():
    """test/testLib_RelativisticElectrons.f90 at 150 kV."""
    e = golden_data.electrons_kat()
    L = O.lib()
    assert "%.8f" % L.oc_wavelength(O._d(e["V"])) == "%.8f" % e["wavelength"]
    assert "%.8f" % L.oc_velocity(O._d(e["V"])) == "%.8f" % e["velocity"]


@pytest.mark.parametrize("sg", [0.0, 0.00745, -0.01])
def test_integrator_perfect_crystal(sg):
    """intensityAtDepthZ (Lib_DiffractionConditions.f90:1209-1259): with x = 1 and
    rho = 1 the RK4 column integrator matches the analytic two-beam intensity."""
    xi0, xig, depth = 113.88929, 308.24709, 0.79 * 96
    a = 2 * np.pi * sg
    want = O.lib().oc_intensity_at_depth(O._d(xi0), O._d(xig), O._d(sg), O._d(depth))
    errs = []
    for nz in (96, 192):
        field = np.ones(nz + 1, dtype=np.complex128)
        rho = np.ones(nz + 1)
        errs.append(abs(O.integrate_column(a, np.pi / xi0, np.pi / xig, depth / nz, field, rho) - want))
    assert errs[0] < 1e-6
    # classic RK4 over double steps: halving dz divides the error by about 16
    assert errs[1] < errs[0] / 10


def test_oracle_thread_count_invariance():
    """The pixel loop is per column: the image does not depend on the thread count."""
    g = golden_data.w_loop()
    args = O.make_args(g["a_super"], 3.1652, (0, 0, 1), (2, 0, 0), R=g["RU"], U=np.eye(3), d=g["d"],
                       xi0=g["xi0"], xig=g["xig"], density=True)
    state, x, _ = O.setup(args, g["pos"])
    G, aa = O.geometry(state, len(x))
    a, _ = O.patch_image(G, aa, x, rows=(10, 20), nthreads=1)
    b, _ = O.patch_image(G, aa, x, rows=(10, 20), nthreads=3)
    assert np.array_equal(a, b)
    assert np.abs(a[:, 10:20]).max() > 0 and np.abs(a[:, :10]).max() == 0
