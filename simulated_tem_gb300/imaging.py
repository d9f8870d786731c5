"""Python API over libstem, shaped like the reference's Fortran interfaces.

* ``DynamicalTwoBeamImaging`` mirrors ``type(DynamicalTwoBeamImaging)`` and its
  public procedures (src/Lib_DynamicalTwoBeamImaging.f90:31-48); its
  ``compute_d2bi_img`` runs ``computeD2BI_img`` on the GPU.
* ``Context`` owns the device buffers (``st_ctx``) and exposes the image and
  blur entry points of include/stem.h.
* ``d2bi_condition`` follows src/d2bi.f90 for one diffraction condition: the
  periodic wrap of the input atoms, the image box from the atom extents, the
  tilt (``-sg``, ``-R``/``-U`` or the default s_g = 0) and the tomography tilt.

Arrays follow the reference's layouts: positions are an (N, 3) C-contiguous
array (the Fortran (3, N) array in memory), images are (Mx, My) arrays in
Fortran order (the reference's column-major d2big2).
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import StGeom, StStats, check, lib

_d = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)


def _cm(m):
    """3x3 matrix -> column-major ctypes double[9]."""
    a = np.asarray(m, dtype=np.float64).reshape(3, 3).ravel(order="F")
    return (_d * 9)(*a)


def _v3(v):
    return (_d * 3)(*[float(t) for t in v])


def _from_cm(arr):
    return np.array(list(arr), dtype=np.float64).reshape(3, 3, order="F")


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Context:
    """A libstem context on one CUDA device (st_create / st_destroy)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().st_create(ctypes.byref(h), device))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            lib().st_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, code):
        check(code, self.handle)

    def image(self, geom, x, aa, flags=0):
        """st_image from host memory: x (N, 3) or (N, ldx) float64; returns the (Mx, My) image (Fortran order)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n, ldx = (x.shape[0], x.shape[1]) if x.ndim == 2 else (0, 3)
        aa = np.ascontiguousarray(np.atleast_1d(aa), dtype=np.float64)
        img = np.zeros((geom.Mx, geom.My), order="F")
        self._check(lib().st_image(self.handle, ctypes.byref(geom), _ptr(x), ldx, n, _ptr(aa), len(aa), flags,
                                   _ptr(img)))
        return img

    def image_device(self, geom, x_dev_ptr, n_atoms, aa, flags, img_dev_ptr, stream=0, ldx=3):
        """st_image_device on device pointers (ints, e.g. torch tensor.data_ptr())."""
        aa = np.ascontiguousarray(np.atleast_1d(aa), dtype=np.float64)
        self._check(lib().st_image_device(self.handle, ctypes.byref(geom), ctypes.c_void_p(x_dev_ptr), ldx, n_atoms,
                                          _ptr(aa), len(aa), flags, ctypes.c_void_p(img_dev_ptr),
                                          ctypes.c_void_p(stream)))

    def image_device_masked(self, geom, x_dev_ptr, n_atoms, aa, flags, img_dev_ptr, mask_dev_ptr, mask_T, stream=0,
                            ldx=3):
        """st_image_device_masked: only the mask_T x mask_T tiles whose mask byte is nonzero."""
        aa = np.ascontiguousarray(np.atleast_1d(aa), dtype=np.float64)
        self._check(lib().st_image_device_masked(self.handle, ctypes.byref(geom), ctypes.c_void_p(x_dev_ptr), ldx,
                                                 n_atoms, _ptr(aa), len(aa), flags, ctypes.c_void_p(img_dev_ptr),
                                                 ctypes.c_void_p(mask_dev_ptr), int(mask_T), ctypes.c_void_p(stream)))

    @staticmethod
    def _job_array(jobs):
        """(geom, x, n_atoms, aa, img[, ldx]) tuples -> st_job array (+ the arrays it points into)."""
        arr = (_lib.StJob * len(jobs))()
        keep = []
        for k, job in enumerate(jobs):
            geom, xp, n, aa, ip = job[:5]
            ldx = job[5] if len(job) > 5 else 3
            aa = np.ascontiguousarray(np.atleast_1d(aa), dtype=np.float64)
            keep.append((geom, aa))
            arr[k].geom = ctypes.pointer(geom)
            arr[k].x = xp
            arr[k].ldx = ldx
            arr[k].nAtoms = n
            arr[k].aa = _ptr(aa)
            arr[k].nPrec = len(aa)
            arr[k].img = ip
        return arr, keep

    def batch_device(self, jobs, flags, stream=0):
        """st_batch_device: jobs is a list of (geom, x_dev_ptr, n_atoms, aa, img_dev_ptr[, ldx])."""
        arr, keep = self._job_array(jobs)
        self._check(lib().st_batch_device(self.handle, len(jobs), arr, flags, ctypes.c_void_p(stream)))

    def plan(self, jobs, flags, stream=0):
        """st_plan_create over (geom, x_dev_ptr, n_atoms, aa, img_dev_ptr[, ldx]) jobs; see Plan."""
        return Plan(self, jobs, flags, stream)

    def batch(self, specs, flags=0):
        """st_batch from host arrays: specs is a list of (geom, x (N, 3) or (N, ldx), aa); returns the images.
        Specs that pass the same x array share one device copy of it."""
        xs, imgs, jobs = {}, [], []
        for geom, x, aa in specs:
            if id(x) not in xs:
                xs[id(x)] = np.ascontiguousarray(x, dtype=np.float64)
            xc = xs[id(x)]
            n, ldx = (xc.shape[0], xc.shape[1]) if xc.ndim == 2 else (0, 3)
            img = np.zeros((geom.Mx, geom.My), order="F")
            imgs.append(img)
            jobs.append((geom, xc.ctypes.data, n, aa, img.ctypes.data, ldx))
        arr, keep = self._job_array(jobs)
        self._check(lib().st_batch(self.handle, len(jobs), arr, flags))
        return imgs

    def blur(self, img, t):
        """st_blur: gaussianBlurImage of an (Nx, Ny) image with width t pixels."""
        img = np.asfortranarray(img, dtype=np.float64)
        out = np.zeros_like(img, order="F")
        self._check(lib().st_blur(self.handle, _ptr(img), img.shape[0], img.shape[1], float(t), _ptr(out)))
        return out

    def blur_device(self, in_ptr, nx, ny, t, out_ptr, stream=0):
        self._check(lib().st_blur_device(self.handle, ctypes.c_void_p(in_ptr), nx, ny, float(t),
                                         ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream)))

    def write_dat(self, path, header, img):
        """st_write_dat: d2bi's .dat file of an (Nx, Ny) image; `header` a dict of
        dat_header() fields or an StDatHeader."""
        img = np.asfortranarray(img, dtype=np.float64)
        h = header if isinstance(header, _lib.StDatHeader) else dat_header(**header)
        self._check(lib().st_write_dat(self.handle, os.fsencode(path), ctypes.byref(h), _ptr(img), img.shape[0],
                                       img.shape[1]))

    def write_png(self, path, img, iso_min=0.0, iso_max=0.0, blur_t=0.0):
        """st_write_png: d2bi's 16-bit PNG of an (Nx, Ny) image (normalised when iso_min ==
        iso_max, else scaled to that window), blurred first when blur_t > 0 pixels."""
        img = np.asfortranarray(img, dtype=np.float64)
        self._check(lib().st_write_png(self.handle, os.fsencode(path), _ptr(img), img.shape[0], img.shape[1],
                                       float(iso_min), float(iso_max), float(blur_t)))

    def png_levels_device(self, img_ptr, nx, ny, levels_ptr, iso_min=0.0, iso_max=0.0, stream=0):
        """st_png_levels_device: nx * ny uint16 levels (x fastest) of a device image."""
        self._check(lib().st_png_levels_device(self.handle, ctypes.c_void_p(img_ptr), nx, ny, float(iso_min),
                                               float(iso_max), ctypes.c_void_p(levels_ptr),
                                               ctypes.c_void_p(stream)))

    def format_dat_device(self, v_ptr, n, text_ptr, cap, stream=0):
        """st_format_dat_device: the '(1000f12.7)' records of n device values."""
        self._check(lib().st_format_dat_device(self.handle, ctypes.c_void_p(v_ptr), int(n),
                                               ctypes.c_void_p(text_ptr), int(cap), ctypes.c_void_p(stream)))

    def read_lammps(self, path, info=None):
        """st_read_lammps: (positions (N, 3), types (N,), header) of a LAMMPS data file, the
        atom lines parsed on the GPU."""
        info = lammps_header(path) if info is None else info
        n = info.n_atoms
        x = np.zeros((n, 3), dtype=np.float64)
        types = np.zeros(n, dtype=np.int32)
        self._check(lib().st_read_lammps(self.handle, os.fsencode(path), ctypes.byref(info), _ptr(x), 3,
                                         ctypes.c_void_p(types.ctypes.data)))
        return x, types, info

    def read_xyz(self, path, info=None, ldx=None):
        """st_read_xyz: (x (N, ldx), types (N,), species names, header) of an .xyz file, the
        atom lines parsed on the GPU; ldx defaults to the file's number of columns."""
        info = xyz_header(path) if info is None else info
        n = max(int(info.n_read), 0)
        ldx = int(info.n_columns) if ldx is None else int(ldx)
        x = np.zeros((n, ldx), dtype=np.float64)
        types = np.zeros(n, dtype=np.int32)
        ns = ctypes.c_int32()
        names = ctypes.create_string_buffer(_lib.ST_XYZ_NAME_LEN * _lib.ST_XYZ_SPECIES_MAX)
        self._check(lib().st_read_xyz(self.handle, os.fsencode(path), ctypes.byref(info), _ptr(x), ldx,
                                      types.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(ns), names,
                                      _lib.ST_XYZ_SPECIES_MAX))
        L = _lib.ST_XYZ_NAME_LEN
        species = [names.raw[L * k:L * k + L].decode("latin-1") for k in range(ns.value)]
        return x, types, species, info

    def parse_xyz_device(self, text_ptr, n_bytes, n_atoms, n_columns, x_ptr, ldx, types_ptr=0, stream=0):
        """st_parse_xyz_device on device buffers: (first bad line or -1, species names)."""
        bad = ctypes.c_int64(-1)
        ns = ctypes.c_int32()
        names = ctypes.create_string_buffer(_lib.ST_XYZ_NAME_LEN * _lib.ST_XYZ_SPECIES_MAX)
        code = lib().st_parse_xyz_device(self.handle, ctypes.c_void_p(text_ptr), int(n_bytes), int(n_atoms),
                                         int(n_columns), ctypes.c_void_p(x_ptr), int(ldx),
                                         ctypes.c_void_p(types_ptr) if types_ptr else None, ctypes.byref(ns), names,
                                         _lib.ST_XYZ_SPECIES_MAX, ctypes.byref(bad), ctypes.c_void_p(stream))
        if code != _lib.ST_OK and bad.value < 0:
            self._check(code)
        L = _lib.ST_XYZ_NAME_LEN
        return bad.value, [names.raw[L * k:L * k + L].decode("latin-1") for k in range(ns.value)]

    def parse_atoms_device(self, text_ptr, n_bytes, n_atoms, x_ptr, types_ptr=0, stream=0):
        """st_parse_atoms_device on device buffers; returns the first bad line or -1."""
        bad = ctypes.c_int64(-1)
        code = lib().st_parse_atoms_device(self.handle, ctypes.c_void_p(text_ptr), int(n_bytes), int(n_atoms),
                                           ctypes.c_void_p(x_ptr), 3, ctypes.c_void_p(types_ptr) if types_ptr else None,
                                           ctypes.byref(bad), ctypes.c_void_p(stream))
        if code != _lib.ST_OK and bad.value < 0:
            self._check(code)
        return bad.value

    def tune(self, mode):
        """st_tune: ST_TUNE_AUTO, ST_TUNE_OFF or a forced slab-ring variant (0 .. st_tune_variants() - 1)."""
        self._check(lib().st_tune(self.handle, int(mode)))

    def stats(self):
        s = StStats()
        self._check(lib().st_get_stats(self.handle, ctypes.byref(s)))
        return s


class Plan:
    """A batch recorded as a CUDA graph (st_plan_*): launch() replays it on a stream,
    wait() completes it (recomputing on the eager path after an overflow)."""

    def __init__(self, ctx, jobs, flags, stream=0):
        arr, keep = ctx._job_array(jobs)
        h = ctypes.c_void_p()
        ctx._check(lib().st_plan_create(ctx.handle, len(jobs), arr, flags, ctypes.c_void_p(stream), ctypes.byref(h)))
        self.handle = h

    def _check(self, code):
        if code != _lib.ST_OK:
            raise _lib.StemError(code, lib().st_plan_last_error(self.handle).decode())

    def launch(self, stream=0):
        self._check(lib().st_plan_launch(self.handle, ctypes.c_void_p(stream)))

    def wait(self, stream=0):
        self._check(lib().st_plan_wait(self.handle, ctypes.c_void_p(stream)))

    def stats(self):
        s = StStats()
        self._check(lib().st_plan_stats(self.handle, ctypes.byref(s)))
        return s

    def close(self):
        if self.handle:
            lib().st_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DynamicalTwoBeamImaging:
    """type(DynamicalTwoBeamImaging) with the reference's procedures (host mirror in libstem)."""

    def __init__(self, a_vox, n_vox, a0, k, g, E, mxy, mzz):
        """DynamicalTwoBeamImaging_ctor0(super, latt, a0, k, g, E, mxy, mzz); super = (a_vox, Nx, Ny, Nz)."""
        h = ctypes.c_void_p()
        check(lib().st_d2bi_create(ctypes.byref(h), _cm(a_vox), int(n_vox[0]), int(n_vox[1]), int(n_vox[2]),
                                   float(a0), _v3(k), _v3(g), float(E), int(mxy), int(mzz)))
        self.handle = h
        self.a0 = float(a0)

    def __del__(self):
        try:
            if self.handle:
                lib().st_d2bi_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def set_conventional_unit_cell(self, a_cell):
        check(lib().st_d2bi_set_conventional_unit_cell(self.handle, _cm(a_cell)))

    def set_voxel_supercell_size(self, d):
        check(lib().st_d2bi_set_voxel_supercell_size(self.handle, _v3(d)))

    def set_deviation_parameter(self, sg):
        check(lib().st_d2bi_set_deviation_parameter(self.handle, float(sg)))

    def set_supercell_tilt(self, U=None, R=None):
        """setSupercellTilt0 (no arguments) or setSupercellTilt2(U, R)."""
        if R is None:
            check(lib().st_d2bi_set_supercell_tilt0(self.handle))
        else:
            check(lib().st_d2bi_set_supercell_tilt2(self.handle, _cm(np.eye(3) if U is None else U), _cm(R)))

    def set_lattice(self, lattice):
        """type(Lattice) of the crystal: "sc", "bcc" (the default), "fcc" or "hcp"."""
        check(lib().st_d2bi_set_lattice(self.handle, _lib.ST_LATTICES[lattice]))

    def set_supercell_tilt_ng(self, ctx, ng, xifile, theta_max=5.0, rho_max=10.0, d_x=0, n_atoms=0, ldx=3):
        """setSupercellTilt1a(ng, xifile [, x]): the -ng tilt search, its scores on the GPU.
        d_x: 0, or the device pointer of the atoms (ldx, n_atoms) for the foil thickness from
        the atoms (-surf).  Returns what the search did (a dict)."""
        info = _lib.StTiltInfo()
        ctx._check(lib().st_d2bi_set_supercell_tilt1a(self.handle, ctx.handle, float(ng), xifile.encode(),
                                                      float(theta_max), float(rho_max), ctypes.c_void_p(d_x),
                                                      int(ldx), int(n_atoms), ctypes.byref(info)))
        return _tilt_info(info)

    def set_extinction_distances(self, xi0, xig):
        check(lib().st_d2bi_set_extinction_distances(self.handle, float(xi0), float(xig)))

    def set_use_density_field(self, use):
        check(lib().st_d2bi_set_use_density_field(self.handle, int(bool(use))))

    def find_image_parameters(self):
        """(aperpx, xmax[3], modg, Mx, My, Mz)."""
        ap, mg = _d(), _d()
        xm = (_d * 3)()
        mx, my, mz = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(lib().st_d2bi_find_image_parameters(self.handle, ctypes.byref(ap), xm, ctypes.byref(mg),
                                                  ctypes.byref(mx), ctypes.byref(my), ctypes.byref(mz)))
        return ap.value, list(xm), mg.value, mx.value, my.value, mz.value

    def get_rotation(self):
        U, R = (_d * 9)(), (_d * 9)()
        check(lib().st_d2bi_get_rotation(self.handle, U, R))
        return _from_cm(U), _from_cm(R)

    def get_deviation_parameter(self):
        return lib().st_d2bi_get_deviation_parameter(self.handle)

    def image_geometry(self, n_atoms, prec_angle=0.005, n_prec=1, nprocs=1, jj=0):
        """The computeD2BI_img prologue: (st_geom, aa[n_prec]) for patch jj of nprocs."""
        G = StGeom()
        aa = np.zeros(n_prec)
        check(lib().st_d2bi_image_geometry(self.handle, int(n_atoms), int(nprocs), int(jj), float(prec_angle),
                                           int(n_prec), ctypes.byref(G), _ptr(aa)))
        return G, aa

    def window_geometry(self, n_atoms, ix0, iy0, dx, dy, prec_angle=0.005, n_prec=1):
        """(st_geom, aa) of the pixel window [ix0, ix0 + dx) x [iy0, iy0 + dy)."""
        G = StGeom()
        aa = np.zeros(n_prec)
        check(lib().st_d2bi_window_geometry(self.handle, int(n_atoms), int(ix0), int(iy0), int(dx), int(dy),
                                            float(prec_angle), int(n_prec), ctypes.byref(G), _ptr(aa)))
        return G, aa

    def compute_d2bi_img(self, ctx, x, prec_angle=0.005, n_prec=1, flags=0):
        """computeD2BI_img on one process: the precession-averaged dark-field image (Mx, My)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        _, _, _, Mx, My, _ = self.find_image_parameters()
        img = np.zeros((Mx, My), order="F")
        check(lib().st_d2bi_compute_img(self.handle, ctx.handle, _ptr(x), x.shape[1], x.shape[0], float(prec_angle),
                                        int(n_prec), int(flags), _ptr(img)), ctx.handle)
        return img


def dat_header(version="1.1.6", k=(0, 0, 1), g=(1, 1, 0), modg=0.0, M=(4, 4), V=200.0, xi0=103.889565,
               xig=207.531624, ng=None, sg=0.0, xmax=(0, 0, 0), aperpx=1.0, rotation=np.eye(3), miller4=False):
    """An StDatHeader from the fields d2bi writes (rotation: the 3 x 3 matrix matmul(R, U))."""
    h = _lib.StDatHeader()
    h.version = version.encode()[:31]
    h.miller4 = 1 if miller4 else 0
    for i, v in enumerate(k):
        h.k[i] = v
    for i, v in enumerate(g):
        h.g[i] = v
    h.modg = modg
    h.nM = len(M)
    for i, v in enumerate(M):
        h.M[i] = int(v)
    h.V, h.xi0, h.xig = V, xi0, xig
    h.has_ng = 0 if ng is None else 1
    h.ng = 0.0 if ng is None else ng
    h.sg = sg
    for i, v in enumerate(xmax):
        h.xmax[i] = v
    h.aperpx = aperpx
    rot = np.asarray(rotation, dtype=np.float64)
    for i, v in enumerate(rot.reshape(-1) if rot.ndim == 1 else rot.T.reshape(-1)):  # column-major
        h.rotation[i] = v
    return h


def format_dat_header(header, nx, ny):
    """st_format_dat_header: the .dat header and size lines (str)."""
    h = header if isinstance(header, _lib.StDatHeader) else dat_header(**header)
    buf = ctypes.create_string_buffer(4096)
    n = ctypes.c_int64(0)
    _lib.check(lib().st_format_dat_header(ctypes.byref(h), nx, ny, buf, 4096, ctypes.byref(n)))
    return buf.raw[:n.value].decode()


def encode_png16(levels):
    """st_encode_png16: a 16-bit greyscale PNG (bytes) of levels [row y, column x]."""
    lv = np.ascontiguousarray(levels, dtype=np.uint16)
    ny, nx = lv.shape
    cap = lib().st_png16_bytes(nx, ny)
    out = ctypes.create_string_buffer(int(cap))
    n = ctypes.c_int64(0)
    _lib.check(lib().st_encode_png16(ctypes.c_void_p(lv.ctypes.data), nx, ny, out, cap, ctypes.byref(n)))
    return out.raw[:n.value]


def lammps_header(path):
    """st_lammps_header: the StLammpsInfo of a LAMMPS data file (n_atoms, n_types, lo, hi,
    data_offset)."""
    info = _lib.StLammpsInfo()
    code = lib().st_lammps_header(os.fsencode(path), ctypes.byref(info))
    if code != _lib.ST_OK:
        raise _lib.StemError(code, "cannot read the LAMMPS header of %s" % path)
    return info


def xyz_header(path):
    """st_xyz_header: the StXyzInfo of an .xyz file (counts, columns, the supercell)."""
    info = _lib.StXyzInfo()
    code = lib().st_xyz_header(os.fsencode(path), ctypes.byref(info))
    if code != _lib.ST_OK:
        raise _lib.StemError(code, "cannot read the .xyz header of %s" % path)
    return info


def fortran_parse_real(text):
    """The reference's ParseReal of a string (None when no number is found)."""
    b = text.encode("latin-1")
    out = ctypes.c_double()
    ok = ctypes.c_int32()
    check(lib().st_fortran_parse_real(b, len(b), ctypes.byref(out), ctypes.byref(ok)))
    return out.value if ok.value else None


def voxel_supercell(a_super, M, a0):
    """d2bi's voxel supercell of the input cell (src/d2bi.f90:856-866): (a_vox, n)."""
    a_super = np.asarray(a_super, dtype=np.float64)
    n = [max(3, int(np.floor(M[0] * _norm2(a_super[:, 0]) / a0))),
         max(3, int(np.floor(M[0] * _norm2(a_super[:, 1]) / a0))),
         max(3, int(np.floor(M[1] * _norm2(a_super[:, 2]) / a0)))]
    a_vox = np.stack([a_super[:, i] / n[i] for i in range(3)], axis=1)
    return a_vox, n


def wrap_pbc(a_super, M, a0, x):
    """d2bi's periodic wrap of the input atoms on the voxel supercell (src/d2bi.f90:856-866); returns a copy."""
    a_vox, n = voxel_supercell(a_super, M, a0)
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    check(lib().st_wrap_pbc(_cm(a_vox), n[0], n[1], n[2], _ptr(x), x.shape[1], x.shape[0]))
    return x, a_vox, n


def _norm2(v):
    """gfortran NORM2 (scaled sum of squares) of a 3-vector."""
    scale, res = 0.0, 1.0
    for t in v:
        t = float(t)
        if t != 0.0:
            ax = abs(t)
            if scale < ax:
                val = scale / ax
                res = 1.0 + res * val * val
                scale = ax
            else:
                val = ax / scale
                res += val * val
    return float(np.sqrt(res)) * scale


def atom_extents(k, g, a_cell, x):
    d = (_d * 3)()
    x = np.ascontiguousarray(x, dtype=np.float64)
    check(lib().st_atom_extents(_v3(k), _v3(g), _cm(a_cell), _ptr(x), x.shape[1], x.shape[0], d))
    return list(d)


def tomography_tilt(tomo_angle, nn, n_tomo, R0):
    R = (_d * 9)()
    check(lib().st_tomography_tilt(float(tomo_angle), int(nn), int(n_tomo), _cm(R0), R))
    return _from_cm(R)


def _tilt_info(info):
    return {name: getattr(info, name) for name, _ in _lib.StTiltInfo._fields_}


def read_extinction_distances(path, hkl, lattice="bcc"):
    """readExtinctionDistance (src/Lib_ReadExtinctionDistances.f90:29-109): (xi_g (n,),
    status 1 all found / 0 some missing / -1 no file)."""
    h = np.ascontiguousarray(hkl, dtype=np.int32).reshape(-1, 3)
    xi = np.zeros(len(h))
    st = ctypes.c_int32()
    symm = _lib.ST_SYMMETRY_HEXAGONAL if lattice == "hcp" else _lib.ST_SYMMETRY_CUBIC
    check(lib().st_read_extinction_distances(path.encode(), len(h), h.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                             symm, _ptr(xi), ctypes.byref(st)))
    return xi, st.value


def permitted_reflections(lattice, rho=10.0):
    """permittedReflections (src/Lib_Lattices.f90:678-735): (n, 3) int32 in the reference's order."""
    n = ctypes.c_int32()
    L = lib()
    check(L.st_permitted_reflections(_lib.ST_LATTICES[lattice], float(rho), None, 0, ctypes.byref(n)))
    h = np.zeros((n.value, 3), dtype=np.int32)
    check(L.st_permitted_reflections(_lib.ST_LATTICES[lattice], float(rho),
                                     h.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), n.value, ctypes.byref(n)))
    return h


def find_best_rotation(ctx, v, z0, a_cell, lattice, hkl, xifile, foil, theta_max=5.0, rho_max=10.0):
    """findBestRotationMatrix (src/Lib_DiffractionConditions.f90:129-357) with the scores on
    the GPU: (U, R, info dict)."""
    U, R = (_d * 9)(), (_d * 9)()
    info = _lib.StTiltInfo()
    h = (ctypes.c_int32 * 3)(*[int(t) for t in hkl])
    ctx._check(lib().st_find_best_rotation(ctx.handle, float(v), _v3(z0), _cm(a_cell), _lib.ST_LATTICES[lattice], h,
                                           xifile.encode(), float(foil), float(theta_max), float(rho_max), U, R,
                                           ctypes.byref(info)))
    return _from_cm(U), _from_cm(R), _tilt_info(info)


def tilt_scores(ctx, v, khat, ghkl, xi_g, foil):
    """The scores of incident vectors khat (nk, 3) against reflections ghkl (nn, 3) with
    extinction distances xi_g (nn,), on the GPU (the first two reflections are not scored)."""
    khat = np.ascontiguousarray(khat, dtype=np.float64)
    ghkl = np.ascontiguousarray(ghkl, dtype=np.float64)
    xi_g = np.ascontiguousarray(xi_g, dtype=np.float64)
    out = np.zeros(len(khat))
    ctx._check(lib().st_tilt_scores(ctx.handle, float(v), _ptr(khat), len(khat), _ptr(ghkl), _ptr(xi_g), len(ghkl),
                                    float(foil), _ptr(out)))
    return out


def tilt_screen(ctx, v, khat, ghkl, xi_g, foil):
    """The FP32 screen of tilt_scores: (scores, bounds on their errors)."""
    khat = np.ascontiguousarray(khat, dtype=np.float64)
    ghkl = np.ascontiguousarray(ghkl, dtype=np.float64)
    xi_g = np.ascontiguousarray(xi_g, dtype=np.float64)
    s, b = np.zeros(len(khat)), np.zeros(len(khat))
    ctx._check(lib().st_tilt_screen(ctx.handle, float(v), _ptr(khat), len(khat), _ptr(ghkl), _ptr(xi_g), len(ghkl),
                                    float(foil), _ptr(s), _ptr(b)))
    return s, b


def d2bi_condition(a_super, a0, k, g, x, V=200.0, M=(4, 4), sg=None, R=None, U=None, d=None, xi0=103.889565,
                   xig=207.533203, density=False, n_tomo=1, tomo_angle=20.0, tomo_step=0, ng=None, xifile=None,
                   lattice="bcc", surf=False, theta_max=5.0, rho_max=10.0, ctx=None):
    """One diffraction condition of the d2bi program (src/d2bi.f90:782-991, 1145-1381).

    Returns (imaging, wrapped positions (N, 3), aperpx).  ``a0`` is the cubic
    lattice constant (``-a0``); a bcc/fcc/sc conventional cell a0 * I is used.
    ``ng`` selects the -ng tilt search (needs ``xifile`` and a GPU context ``ctx``;
    ``surf`` takes the foil thickness from the atoms); with ``xifile`` xi0 and xig are
    the table's values for [000] and g (:1183-1192).
    """
    a0 = (a0 + a0 + a0) / 3  # a0 = (a0in(1) + a0in(2) + a0in(3)) / 3 (:787-788)
    xw, a_vox, n = wrap_pbc(a_super, M, a0, x)
    a_cell = a0 * np.eye(3)
    if d is None:
        d = atom_extents(k, g, a_cell, xw)
    d_x = None
    if ng is not None and surf:
        import torch
        d_x = torch.from_numpy(np.ascontiguousarray(xw)).to("cuda")
    t = _condition(a_vox, n, a0, k, g, d, V, M, sg, R, U, xi0, xig, density, n_tomo, tomo_angle, tomo_step,
                   ng=ng, xifile=xifile, lattice=lattice, theta_max=theta_max, rho_max=rho_max, ctx=ctx,
                   d_x=0 if d_x is None else d_x.data_ptr(), n_atoms=len(xw))
    return t, xw, t.aperpx


def _condition(a_vox, n, a0, k, g, d, V, M, sg, R, U, xi0, xig, density, n_tomo, tomo_angle, tomo_step, ng=None,
               xifile=None, lattice="bcc", theta_max=5.0, rho_max=10.0, ctx=None, d_x=0, n_atoms=0):
    """The imaging set-up of one condition on already wrapped atoms with extents d."""
    a_cell = a0 * np.eye(3)
    if xifile:
        gi = [int(np.copysign(np.floor(abs(v) + 0.5), v)) for v in g]  # nint: halves away from zero
        xi, status = read_extinction_distances(xifile, [[0, 0, 0], gi], lattice)
        if status != 1:
            raise _lib.StemError(_lib.ST_ERR_ARG, "no xi_g for [000] and g in %s" % xifile)
        xi0, xig = float(xi[0]), float(xi[1])
    t = DynamicalTwoBeamImaging(a_vox, n, a0, k, g, V, M[0], M[1])
    t.set_conventional_unit_cell(a_cell)
    t.set_lattice(lattice)
    t.set_voxel_supercell_size(d)
    t.tilt = None
    if ng is not None:
        if ctx is None or not xifile:
            raise _lib.StemError(_lib.ST_ERR_ARG, "the -ng tilt search needs xifile and a GPU context")
        t.tilt = t.set_supercell_tilt_ng(ctx, ng, xifile, theta_max, rho_max, d_x, n_atoms)
    elif sg is not None:
        t.set_deviation_parameter(sg)
        t.set_supercell_tilt()
    elif R is not None:
        t.set_supercell_tilt(np.eye(3) if U is None else U, R)
    else:
        t.set_deviation_parameter(0.0)
        t.set_supercell_tilt()
    U0, R0 = t.get_rotation()
    t.set_extinction_distances(xi0, xig)
    t.aperpx = t.find_image_parameters()[0]
    t.set_use_density_field(density)
    if n_tomo > 1:
        t.set_supercell_tilt(U0, tomography_tilt(tomo_angle, tomo_step, n_tomo, R0))
    return t


def d2bi_sweep(ctx, a_super, a0, k, gs, x, n_tomo=1, tomo_angle=20.0, prec_angle=0.0, n_prec=1, V=200.0, M=(4, 4),
               sg=None, xi0=103.889565, xig=207.533203, density=False, stream=0):
    """The conditions of a d2bi sweep (g-vectors gs x tomography steps) with the passes over
    the atoms on the GPU: the atoms are wrapped once in device memory (st_wrap_pbc_device)
    and the extents of every g come from one pass (st_atom_extents_device); the per-image
    set-up is scalar host work.  Returns (wrapped positions: a torch device tensor (N, 3),
    [(geometry, aa)] in g-major order, the imaging objects).  The geometries equal those of
    d2bi_condition for each (g, step), bit for bit."""
    import torch
    a0 = (a0 + a0 + a0) / 3
    a_vox, n = voxel_supercell(a_super, M, a0)
    x = np.ascontiguousarray(x, dtype=np.float64)
    d_x = torch.from_numpy(x).to("cuda").contiguous()
    ctx._check(lib().st_wrap_pbc_device(ctx.handle, _cm(a_vox), n[0], n[1], n[2], ctypes.c_void_p(d_x.data_ptr()),
                                        3, len(x), ctypes.c_void_p(stream)))
    a_cell = a0 * np.eye(3)
    gs = [tuple(g) for g in gs]
    nc = len(gs)
    ks = (_d * (3 * nc))(*[float(v) for _ in gs for v in k])
    gv = (_d * (3 * nc))(*[float(v) for g in gs for v in g])
    dd = (_d * (3 * nc))()
    if stream:
        torch.cuda.current_stream().synchronize()
    ctx._check(lib().st_atom_extents_device(ctx.handle, nc, ks, gv, _cm(a_cell), ctypes.c_void_p(d_x.data_ptr()),
                                            3, len(x), dd))
    specs, conds = [], []
    for c, g in enumerate(gs):
        d = [dd[3 * c], dd[3 * c + 1], dd[3 * c + 2]]
        for step in range(n_tomo):
            t = _condition(a_vox, n, a0, k, g, d, V, M, sg, None, None, xi0, xig, density, n_tomo, tomo_angle,
                           step)
            G, aa = t.image_geometry(len(x), prec_angle=prec_angle, n_prec=n_prec)
            specs.append((G, aa))
            conds.append(t)
    return d_x, specs, conds
