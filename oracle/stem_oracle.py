"""ORACLE -- test infrastructure only.

ctypes binding of ``libstem_oracle.so``, the plain-C restatement of the
reference's imaging path (``stem_oracle.c``).  Only the tests, the smoke check
and the CPU-baseline leg of the benchmark import this module, always as the
checker; the product path never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstem_oracle.so")

_d = ctypes.c_double
_i = ctypes.c_int
_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Super(ctypes.Structure):
    _fields_ = [("Nx", _i), ("Ny", _i), ("Nz", _i), ("a", _d * 9), ("ia", _d * 9)]


class D2BI(ctypes.Structure):
    _fields_ = [("k", _d * 3), ("g", _d * 3), ("a0", _d), ("super", Super), ("sg", _d), ("mxy", _i), ("mzz", _i),
                ("xi0", _d), ("xig", _d), ("E", _d), ("useDensityField", _i), ("gksuper", Super), ("delta", _d * 3),
                ("foilThickness", _d), ("voxelSupercellDimensions", _d * 3), ("nuvw", _i), ("uvw", _i * 375),
                ("a_cell", _d * 9), ("U", _d * 9), ("R", _d * 9), ("test", _i)]


class Geom(ctypes.Structure):
    _fields_ = [("Mx", _i), ("My", _i), ("Mz", _i), ("ix0", _i), ("ix1", _i), ("iy0", _i), ("iy1", _i),
                ("Ex", _i), ("Ey", _i), ("Ez", _i), ("deltaM", _i), ("nMax0", _i), ("nuvw", _i),
                ("RU", _d * 9), ("delta", _d * 3), ("Ruvw", _d * 81), ("lc_delta", _d * 3), ("a_col", _d * 9),
                ("ia_col", _d * 9), ("a_vox", _d * 9), ("g", _d * 3), ("sigma", _d), ("cut2", _d), ("i2s2", _d),
                ("deltaz", _d), ("b0", _d), ("bg", _d), ("useDensity", _i)]


class Stats(ctypes.Structure):
    _fields_ = [("n_kept", _i64), ("n_tests", _i64), ("n_accepted", _i64), ("n_voxels", _i64),
                ("max_cell_count", _i)]


class Args(ctypes.Structure):
    _fields_ = [("a_super", _d * 9), ("a0in", _d), ("k", _d * 3), ("g", _d * 3), ("V", _d), ("M", _i * 2),
                ("tilt_mode", _i), ("sg", _d), ("haveU", _i), ("U", _d * 9), ("R", _d * 9), ("haveD", _i),
                ("d0", _d * 3), ("xi0", _d), ("xig", _d), ("useDensity", _i), ("nPrec", _i), ("precAngle", _d),
                ("nTomo", _i), ("tomoAngle", _d), ("dark", _i), ("ng", _d), ("lattice", _i), ("surf", _i),
                ("thetaMax", _d), ("rhoMax", _d), ("xifile", ctypes.c_char * 512)]


class TiltInfo(ctypes.Structure):
    _fields_ = [("nk", _i), ("nn", _i), ("ii_best", _i), ("attempt", _i), ("xi_ok", _i), ("ss_best", _d),
                ("theta", _d), ("phi", _d), ("foil", _d), ("foil_sigma", _d), ("dark_theta", _d)]


LATTICES = {"custom": 0, "sc": 1, "bcc": 2, "fcc": 3, "hcp": 4}


_lib = None


def build():
    """Compile the oracle with its Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oc_norm2.restype = _d
        L.oc_wavelength.restype = _d
        L.oc_velocity.restype = _d
        L.oc_intensity_at_depth.restype = _d
        L.oc_integrate_column.restype = _d
        L.oc_get_deviation_parameter.restype = _d
        L.oc_score_incident_vector.restype = _d
        for name in ("oc_image_geometry", "oc_patch_image", "oc_patch_image_rows", "oc_compute_d2bi_img",
                     "oc_neighbour_list", "oc_d2bi_setup"):
            getattr(L, name).restype = _i
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _mat(m):
    """3x3 numpy (row i, column j) -> column-major ctypes array."""
    m = np.asarray(m, dtype=np.float64)
    return (_d * 9)(*m.T.reshape(-1))


def make_args(a_super, a0, k, g, V=200.0, M=(4, 4), sg=None, R=None, U=None, d=None, xi0=103.889565,
              xig=207.533203, density=False, nPrec=1, precAngle=0.005, nTomo=1, tomoAngle=20.0, dark=True, ng=None,
              xifile=None, lattice="bcc", surf=False, theta_max=5.0, rho_max=10.0):
    """d2bi command-line arguments for one diffraction condition (src/d2bi.f90:48-100 defaults)."""
    a = Args()
    a.a_super[:] = list(np.asarray(a_super, dtype=np.float64).T.reshape(-1))
    a.a0in = a0
    a.k[:] = list(map(float, k))
    a.g[:] = list(map(float, g))
    a.V = V
    a.M[:] = list(M)
    a.lattice = LATTICES[lattice]
    a.thetaMax, a.rhoMax = theta_max, rho_max
    a.surf = int(bool(surf))
    if xifile:
        a.xifile = xifile.encode()
    if ng is not None:
        a.tilt_mode = 3
        a.ng = ng
    elif R is not None:
        a.tilt_mode = 2
        a.R[:] = list(np.asarray(R, dtype=np.float64).T.reshape(-1))
        if U is not None:
            a.haveU = 1
            a.U[:] = list(np.asarray(U, dtype=np.float64).T.reshape(-1))
    elif sg is not None:
        a.tilt_mode = 1
        a.sg = sg
    else:
        a.tilt_mode = 0
    if d is not None:
        a.haveD = 1
        a.d0[:] = list(map(float, d))
    a.xi0, a.xig = xi0, xig
    a.useDensity = int(bool(density))
    a.nPrec, a.precAngle = nPrec, precAngle
    a.nTomo, a.tomoAngle = nTomo, tomoAngle
    a.dark = int(bool(dark))
    return a


def setup(args, pos, nn=0):
    """wrapPBC the atoms and set up the imaging state; returns (state, wrapped x (N,3), aperpx)."""
    x = np.ascontiguousarray(pos, dtype=np.float64).copy()
    t = D2BI()
    aperpx = _d()
    rc = lib().oc_d2bi_setup(ctypes.byref(args), _dptr(x), _i64(3), _i64(x.shape[0]), _i(nn), ctypes.byref(t),
                             ctypes.byref(aperpx))
    if rc != 0:
        raise RuntimeError("oracle setup failed: %d" % rc)
    return t, x, aperpx.value


def geometry(state, n_atoms, nPrec=1, precAngle=0.005, nProcs=1, jj=0):
    G = Geom()
    aa = np.zeros(max(nPrec, 1))
    rc = lib().oc_image_geometry(ctypes.byref(state), _i64(n_atoms), _i(nProcs), _i(jj), _d(precAngle), _i(nPrec),
                                 ctypes.byref(G), _dptr(aa))
    if rc != 0:
        raise RuntimeError("oracle geometry failed: %d" % rc)
    return G, aa


def patch_image(G, aa, x, img=None, rows=None, nthreads=1):
    """Sum over precession of |phi_g|^2 for the pixels of the patch (column-major (Mx, My) in a numpy (Mx, My) array
    stored Fortran-order); returns (img, stats)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    if img is None:
        img = np.zeros((G.Mx, G.My), order="F")
    st = Stats()
    aa = np.ascontiguousarray(aa, dtype=np.float64)
    if rows is None:
        rc = lib().oc_patch_image(ctypes.byref(G), _dptr(aa), _i(len(aa)), _dptr(x), _i64(3), _i64(x.shape[0]),
                                  _dptr(img), ctypes.byref(st), _i(nthreads))
    else:
        rc = lib().oc_patch_image_rows(ctypes.byref(G), _dptr(aa), _i(len(aa)), _dptr(x), _i64(3),
                                       _i64(x.shape[0]), _i(rows[0]), _i(rows[1]), _dptr(img), ctypes.byref(st),
                                       _i(nthreads))
    if rc != 0:
        raise RuntimeError("oracle image failed: %d" % rc)
    return img, st


def compute_d2bi_img(state, x, nPrec=1, precAngle=0.005, nthreads=1):
    """computeD2BI_img: the precession-averaged dark-field image (Mx, My)."""
    Mx, My = state.gksuper.Nx, state.gksuper.Ny
    img = np.zeros((Mx, My), order="F")
    st = Stats()
    x = np.ascontiguousarray(x, dtype=np.float64)
    rc = lib().oc_compute_d2bi_img(ctypes.byref(state), _dptr(x), _i64(3), _i64(x.shape[0]), _d(precAngle),
                                   _i(nPrec), _dptr(img), ctypes.byref(st), _i(nthreads))
    if rc != 0:
        raise RuntimeError("oracle computeD2BI_img failed: %d" % rc)
    return img, st


def integrate_column(a, b0, bg, dz, field, rho):
    f = np.ascontiguousarray(np.stack([field.real, field.imag], axis=-1).reshape(-1))
    r = np.ascontiguousarray(rho, dtype=np.float64)
    return lib().oc_integrate_column(_d(a), _d(b0), _d(bg), _d(dz), _dptr(f), _dptr(r), _i(len(rho) - 1))


def gaussian_blur(img, t):
    img = np.asfortranarray(img, dtype=np.float64)
    out = np.zeros_like(img, order="F")
    lib().oc_gaussian_blur(_dptr(img), _i(img.shape[0]), _i(img.shape[1]), _d(t), _dptr(out))
    return out


def png_levels_window(img, lo, hi):
    """outputImgAsPng's contrast mode: levels of clamp((v - lo) / (hi - lo), 0, 1)."""
    img = np.asfortranarray(img, dtype=np.float64)
    Nx, Ny = img.shape
    lv = np.zeros((Ny, Nx), dtype=np.uint16)
    lib().oc_png_levels_window(_dptr(img), _i(Nx), _i(Ny), _d(lo), _d(hi),
                               lv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
    return lv


def format_f12_7(values):
    """The '(1000f12.7)' records of a .dat file for a flat array of values (bytes)."""
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = ctypes.create_string_buffer(12 * v.size + v.size // 1000 + 2)
    L = lib()
    L.oc_format_f12_7.restype = ctypes.c_longlong
    n = L.oc_format_f12_7(_dptr(v), ctypes.c_longlong(v.size), out)
    return out.raw[:n]


def fortran_f(x, w, d):
    """Fortran Fw.d editing of one number (the .dat header's fields)."""
    if x != x:
        s = "NaN"
    elif x in (float("inf"), float("-inf")):
        s = "Infinity" if x > 0 else "-Infinity"
    else:
        s = "%.*f" % (d, abs(x)) + ("." if d == 0 else "")
        if np.signbit(x):
            s = "-" + s
        if len(s) > w and s.lstrip("-").startswith("0."):
            s = s.replace("0.", ".", 1)
    return "*" * w if len(s) > w else s.rjust(w)


def fortran_i(v, w):
    """Fortran Iw editing."""
    s = "%d" % v
    return "*" * w if len(s) > w else s.rjust(w)


def dat_header(h, nx, ny):
    """The header and size lines of d2bi's .dat file (src/d2bi.f90:1430-1454) for a dict
    of the written fields."""
    nv = 4 if h.get("miller4") else 3
    out = ["# d2bi v." + h["version"],
           "# k       " + "".join(fortran_f(v, 10, 3) for v in h["k"][:nv]),
           "# g       " + "".join(fortran_f(v, 10, 3) for v in h["g"][:nv]) + fortran_f(h["modg"], 12, 5),
           "# M       " + "".join(fortran_i(m, 8) for m in h["M"]),
           "# V (keV) " + fortran_f(h["V"], 10, 0),
           "# xi (A)  " + fortran_f(h["xi0"], 12, 5) + fortran_f(h["xig"], 12, 5)]
    if h.get("ng") is not None:
        out.append("# n_g     " + fortran_f(h["ng"], 8, 3))
    out += ["# s_g (1/A)    " + fortran_f(h["sg"], 12, 5),
            "# img space (A)" + "".join(fortran_f(v, 12, 3) for v in h["xmax"]),
            "# scale (A/px) " + fortran_f(h["aperpx"], 12, 5),
            "# rotation " + "".join(fortran_f(v, 12, 6) for v in h["rotation"]),
            fortran_i(nx, 8) + fortran_i(ny, 8)]
    return "\n".join(out) + "\n"


def read_lammps_atoms(path, offset, n_atoms):
    """input_lammps's atom lines: (positions (n, 3), types (n,)); raises on a bad line."""
    x = np.zeros((n_atoms, 3), dtype=np.float64)
    ty = np.zeros(n_atoms, dtype=np.int32)
    L = lib()
    L.oc_read_lammps_atoms.restype = ctypes.c_longlong
    bad = L.oc_read_lammps_atoms(os.fsencode(path), ctypes.c_longlong(offset), ctypes.c_longlong(n_atoms),
                                 _dptr(x), ty.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if bad:
        raise ValueError("atom line %d does not hold id type x y z" % bad)
    return x, ty


def png_levels(img):
    img = np.asfortranarray(img, dtype=np.float64)
    Nx, Ny = img.shape
    lv = np.zeros((Ny, Nx), dtype=np.uint16)
    lib().oc_png_levels(_dptr(img), _i(Nx), _i(Ny), lv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
    return lv


def neighbour_list(a_cell, cells, nmax0, points, query, cutoff):
    s = Super()
    s.Nx, s.Ny, s.Nz = cells
    s.a[:] = list(np.asarray(a_cell, dtype=np.float64).T.reshape(-1))
    L = lib()
    L.oc_inv3(s.a, s.ia)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    q = np.ascontiguousarray(query, dtype=np.float64)
    maxn = len(points)
    ids = np.zeros(maxn, dtype=np.int32)
    dx = np.zeros((maxn, 3))
    r2 = np.zeros(maxn)
    mc = _i()
    n = L.oc_neighbour_list(ctypes.byref(s), _dptr(pts), _i(len(pts)), _i(nmax0), _dptr(q), _d(cutoff),
                            ids.ctypes.data_as(_ip), _dptr(dx), _dptr(r2), _i(maxn), ctypes.byref(mc))
    if n < 0:
        raise RuntimeError("oracle neighbour list failed: %d" % -n)
    return ids[:n], dx[:n], r2[:n], mc.value


def read_extinction_distances(path, hkl, symm=1):
    """readExtinctionDistance: (xi_g (n,), status 1 / 0 / -1)."""
    hkl = np.ascontiguousarray(hkl, dtype=np.int32).reshape(-1, 3)
    xi = np.zeros(len(hkl))
    rc = lib().oc_read_extinction_distances(path.encode(), hkl.ctypes.data_as(_ip), _i(len(hkl)), _i(symm),
                                            _dptr(xi))
    return xi, rc


def permitted_reflections(lattice, rho=10.0):
    L = lib()
    n = L.oc_permitted_reflections(_i(LATTICES[lattice]), _d(rho), None, _i(0))
    hkl = np.zeros((n, 3), dtype=np.int32)
    L.oc_permitted_reflections(_i(LATTICES[lattice]), _d(rho), hkl.ctypes.data_as(_ip), _i(n))
    return hkl


def find_best_rotation(v, z0, a_cell, lattice, hkl, xifile, foil, theta_max=5.0, rho_max=10.0):
    """findBestRotationMatrix: (U, R, TiltInfo, scores (nk,), khat (nk, 3))."""
    U, R = (_d * 9)(), (_d * 9)()
    info = TiltInfo()
    scores = np.zeros(8000)
    khat = np.zeros((8000, 3))
    h = (_i * 3)(*[int(t) for t in hkl])
    rc = lib().oc_find_best_rotation(_d(v), (_d * 3)(*map(float, z0)), _mat(a_cell), _i(LATTICES[lattice]), h,
                                     xifile.encode(), _d(foil), _d(theta_max), _d(rho_max), U, R,
                                     ctypes.byref(info), _dptr(scores), _dptr(khat))
    if rc != 0:
        raise RuntimeError("oracle tilt search failed: %d" % rc)
    cm = lambda m: np.array(list(m)).reshape(3, 3).T
    return cm(U), cm(R), info, scores[:info.nk].copy(), khat[:info.nk].copy()


def quaternion_round_trip(R):
    """quaternionToRotMat(RotMatToQuaternion(R)) and the quaternion (w, x, y, z)."""
    q = (_d * 4)()
    lib().oc_rotmat_to_quaternion(_mat(R), q)
    out = (_d * 9)()
    lib().oc_quaternion_to_rotmat(q, out)
    return np.array(list(out)).reshape(3, 3).T, np.array(list(q))


def tilt_reflections(lattice, a_cell, hkl, xifile, rho=10.0):
    """The scoring inputs of the tilt search: (ghkl (nn, 3), xi_g (nn,))."""
    h = (_i * 3)(*[int(t) for t in hkl])
    L = lib()
    nn = L.oc_tilt_reflections(_i(LATTICES[lattice]), _mat(a_cell), h, _d(rho), xifile.encode(), None, None, _i(0))
    g = np.zeros((nn, 3))
    xi = np.zeros(nn)
    L.oc_tilt_reflections(_i(LATTICES[lattice]), _mat(a_cell), h, _d(rho), xifile.encode(), _dptr(g), _dptr(xi),
                          _i(nn))
    return g, xi


class XyzInfo(ctypes.Structure):
    _fields_ = [("n_atoms", ctypes.c_longlong), ("n_read", ctypes.c_longlong), ("n_columns", _i),
                ("n_header_lines", _i), ("lammps", _i), ("supercell_kind", _i), ("supercell_ok", _i),
                ("repeats", _i * 3), ("a_super", _d * 9), ("data_offset", ctypes.c_longlong),
                ("file_bytes", ctypes.c_longlong), ("column_description", ctypes.c_char * 257)]


def xyz_header(path):
    info = XyzInfo()
    rc = lib().oc_xyz_header(path.encode(), ctypes.byref(info))
    if rc != 0:
        raise RuntimeError("oracle xyz header failed: %d" % rc)
    return info


def read_xyz_atoms(path, info, ldx=None):
    """input0: (x (n, ldx), types (n,), species names)."""
    n, nc = info.n_read, info.n_columns
    ldx = nc if ldx is None else ldx
    x = np.zeros((n, ldx))
    types = np.zeros(n, dtype=np.int32)
    names = ctypes.create_string_buffer(6 * 1000)
    L = lib()
    L.oc_read_xyz_atoms.restype = ctypes.c_longlong
    rc = L.oc_read_xyz_atoms(path.encode(), ctypes.c_longlong(info.data_offset), ctypes.c_longlong(n), _i(nc),
                             _dptr(x), _i(ldx), types.ctypes.data_as(_ip), names, _i(1000))
    if rc < 0:
        raise RuntimeError("oracle xyz read failed at line %d" % (-rc - 1))
    sp = [names.raw[6 * k:6 * k + 6].decode() for k in range(rc)]
    return x, types, sp


def fortran_parse_real(text):
    r = _d()
    b = text.encode()
    ok = lib().oc_fortran_parse_real(b, _i(len(b)), ctypes.byref(r))
    return (r.value if ok else None)
