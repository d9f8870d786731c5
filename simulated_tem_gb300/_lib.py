"""ctypes binding of libstem.so (include/stem.h, include/stem_host.h).

The library is built in-tree by ``simulated_tem_gb300/build.py``.  There is no
fallback: if the library is missing or does not load, every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstem.so")
PEAKS_PATH = os.path.join(HERE, "libstem_peaks.so")

ST_OK = 0
ST_ERR_ARG = 1
ST_ERR_CAPACITY = 2
ST_ERR_CUDA = 3
ST_ERR_TIMEOUT = 4
ST_ERR_ALLOC = 5

ST_FLAG_FP32 = 0x1
ST_FLAG_AVERAGE = 0x2
ST_FLAG_BRIGHT = 0x4
ST_FLAG_STATS = 0x8
ST_TUNE_AUTO = -1
ST_TUNE_OFF = -2

ST_BLUR_NOALLOC_MAX_PIXELS = 1 << 21
ST_BLUR_NOALLOC_MAX_NX = 4096

_d = ctypes.c_double
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class StGeom(ctypes.Structure):
    """st_geom of include/stem.h."""
    _fields_ = [("RU", _d * 9), ("delta", _d * 3), ("nuvw", _i32), ("pad0", _i32), ("Ruvw", _d * 81),
                ("g", _d * 3), ("a_col", _d * 9), ("ia_col", _d * 9), ("Ex", _i32), ("Ey", _i32), ("Ez", _i32),
                ("nMax0", _i32), ("lc_delta", _d * 3), ("a_vox", _d * 9), ("Mx", _i32), ("My", _i32),
                ("Mz", _i32), ("ix0", _i32), ("ix1", _i32), ("iy0", _i32), ("iy1", _i32), ("useDensity", _i32),
                ("sigma", _d), ("deltaz", _d), ("b0", _d), ("bg", _d)]


class StStats(ctypes.Structure):
    """st_stats of include/stem.h."""
    _fields_ = [("n_atoms", _i64), ("n_kept", _i64), ("n_tests", _i64), ("n_accepted", _i64),
                ("n_voxels", _i64), ("max_cell_count", _i32), ("n_prec", _i32), ("ms_bin", _d),
                ("ms_column", _d), ("column_kernel", _i32), ("ring_variant", _i32), ("ring_slab_atoms", _i32),
                ("n_launches", _i32)]


class StJob(ctypes.Structure):
    """st_job of include/stem.h."""
    _fields_ = [("geom", ctypes.POINTER(StGeom)), ("x", _vp), ("ldx", _i64), ("nAtoms", _i64), ("aa", _dp),
                ("nPrec", _i32), ("pad0", _i32), ("img", _vp)]


class StDatHeader(ctypes.Structure):
    """st_dat_header of include/stem.h (the .dat file's header fields)."""
    _fields_ = [("version", ctypes.c_char * 32), ("miller4", _i32), ("k", _d * 4), ("g", _d * 4), ("modg", _d),
                ("nM", _i32), ("M", _i32 * 3), ("V", _d), ("xi0", _d), ("xig", _d), ("has_ng", _i32), ("ng", _d),
                ("sg", _d), ("xmax", _d * 3), ("aperpx", _d), ("rotation", _d * 9)]


class StLammpsInfo(ctypes.Structure):
    """st_lammps_info of include/stem.h (a LAMMPS data file's header)."""
    _fields_ = [("n_atoms", _i64), ("n_types", _i32), ("pad0", _i32), ("lo", _d * 3), ("hi", _d * 3),
                ("data_offset", _i64), ("file_bytes", _i64)]


class StXyzInfo(ctypes.Structure):
    """st_xyz_info of include/stem.h (an .xyz file's header)."""
    _fields_ = [("n_atoms", _i64), ("n_read", _i64), ("n_columns", _i32), ("n_header_lines", _i32),
                ("lammps", _i32), ("supercell_kind", _i32), ("supercell_ok", _i32), ("repeats", _i32 * 3),
                ("a_super", _d * 9), ("data_offset", _i64), ("file_bytes", _i64),
                ("column_description", ctypes.c_char * 257)]


class StTiltInfo(ctypes.Structure):
    """st_tilt_info of include/stem_host.h (what a -ng tilt search did)."""
    _fields_ = [("nk", _i32), ("nn", _i32), ("ii_best", _i32), ("attempt", _i32), ("xi_status", _i32),
                ("n_recheck", _i32), ("ss_best", _d), ("theta", _d), ("phi", _d), ("foil", _d),
                ("foil_sigma", _d), ("dark_theta", _d), ("scan_ms", _d), ("foil_ms", _d), ("n_fp64", _i32),
                ("pad0", _i32), ("screen_ms", _d)]


ST_LATTICES = {"sc": 1, "bcc": 2, "fcc": 3, "hcp": 4}
ST_XYZ_SPECIES_MAX = 1000
ST_XYZ_NAME_LEN = 6
ST_SYMMETRY_CUBIC = 1
ST_SYMMETRY_HEXAGONAL = 2


class StemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libstem error %d: %s" % (code, msg))
        self.code = code


_PROTOS = {
    # include/stem.h
    "st_create": (_i32, [ctypes.POINTER(_vp), _i32]),
    "st_destroy": (None, [_vp]),
    "st_last_error": (ctypes.c_char_p, [_vp]),
    "st_image": (_i32, [_vp, ctypes.POINTER(StGeom), _dp, _i64, _i64, _dp, _i32, _i32, _dp]),
    "st_image_device": (_i32, [_vp, ctypes.POINTER(StGeom), _vp, _i64, _i64, _dp, _i32, _i32, _vp, _vp]),
    "st_blur": (_i32, [_vp, _dp, _i32, _i32, _d, _dp]),
    "st_blur_device": (_i32, [_vp, _vp, _i32, _i32, _d, _vp, _vp]),
    "st_get_stats": (_i32, [_vp, ctypes.POINTER(StStats)]),
    "st_blur_noalloc": (_i32, [_vp, _i32, _i32, _d, _vp, _vp, ctypes.c_char_p, _i32]),
    "st_batch_device": (_i32, [_vp, _i32, ctypes.POINTER(StJob), _i32, _vp]),
    "st_batch": (_i32, [_vp, _i32, ctypes.POINTER(StJob), _i32]),
    "st_image_device_masked": (_i32, [_vp, ctypes.POINTER(StGeom), _vp, _i64, _i64, _dp, _i32, _i32, _vp, _vp, _i32,
                                      _vp]),
    "st_tune": (_i32, [_vp, _i32]),
    "st_plan_create": (_i32, [_vp, _i32, ctypes.POINTER(StJob), _i32, _vp, ctypes.POINTER(_vp)]),
    "st_plan_launch": (_i32, [_vp, _vp]),
    "st_plan_wait": (_i32, [_vp, _vp]),
    "st_plan_stats": (_i32, [_vp, ctypes.POINTER(StStats)]),
    "st_plan_last_error": (ctypes.c_char_p, [_vp]),
    "st_plan_destroy": (None, [_vp]),
    "st_tune_variants": (_i32, []),
    "st_tune_variant_name": (ctypes.c_char_p, [_i32]),
    "st_format_dat_header": (_i32, [ctypes.POINTER(StDatHeader), _i32, _i32, ctypes.c_char_p, _i64,
                                    ctypes.POINTER(_i64)]),
    "st_dat_text_bytes": (_i64, [_i64]),
    "st_format_dat_device": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "st_write_dat": (_i32, [_vp, ctypes.c_char_p, ctypes.POINTER(StDatHeader), _dp, _i32, _i32]),
    "st_png_levels_device": (_i32, [_vp, _vp, _i32, _i32, _d, _d, _vp, _vp]),
    "st_png16_bytes": (_i64, [_i32, _i32]),
    "st_encode_png16": (_i32, [_vp, _i32, _i32, _vp, _i64, ctypes.POINTER(_i64)]),
    "st_write_png": (_i32, [_vp, ctypes.c_char_p, _dp, _i32, _i32, _d, _d, _d]),
    "st_lammps_header": (_i32, [ctypes.c_char_p, ctypes.POINTER(StLammpsInfo)]),
    "st_parse_real": (_i32, [ctypes.c_char_p, _i64, _dp, ctypes.POINTER(_i32)]),
    "st_parse_atoms_device": (_i32, [_vp, _vp, _i64, _i64, _vp, _i64, _vp, ctypes.POINTER(_i64), _vp]),
    "st_read_lammps": (_i32, [_vp, ctypes.c_char_p, ctypes.POINTER(StLammpsInfo), _dp, _i64, _vp]),
    # include/stem_host.h
    "st_d2bi_create": (_i32, [ctypes.POINTER(_vp), _dp, _i32, _i32, _i32, _d, _dp, _dp, _d, _i32, _i32]),
    "st_d2bi_destroy": (None, [_vp]),
    "st_d2bi_set_conventional_unit_cell": (_i32, [_vp, _dp]),
    "st_d2bi_set_voxel_supercell_size": (_i32, [_vp, _dp]),
    "st_d2bi_set_deviation_parameter": (_i32, [_vp, _d]),
    "st_d2bi_set_supercell_tilt0": (_i32, [_vp]),
    "st_d2bi_set_supercell_tilt2": (_i32, [_vp, _dp, _dp]),
    "st_d2bi_set_extinction_distances": (_i32, [_vp, _d, _d]),
    "st_d2bi_set_use_density_field": (_i32, [_vp, _i32]),
    "st_d2bi_find_image_parameters": (_i32, [_vp, _dp, _dp, _dp, ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                              ctypes.POINTER(_i32)]),
    "st_d2bi_get_rotation": (_i32, [_vp, _dp, _dp]),
    "st_d2bi_get_deviation_parameter": (_d, [_vp]),
    "st_d2bi_image_geometry": (_i32, [_vp, _i64, _i32, _i32, _d, _i32, ctypes.POINTER(StGeom), _dp]),
    "st_d2bi_window_geometry": (_i32, [_vp, _i64, _i32, _i32, _i32, _i32, _d, _i32, ctypes.POINTER(StGeom), _dp]),
    "st_d2bi_compute_img": (_i32, [_vp, _vp, _dp, _i64, _i64, _d, _i32, _i32, _dp]),
    "st_wrap_pbc": (_i32, [_dp, _i32, _i32, _i32, _dp, _i64, _i64]),
    "st_atom_extents": (_i32, [_dp, _dp, _dp, _dp, _i64, _i64, _dp]),
    "st_tomography_tilt": (_i32, [_d, _i32, _i32, _dp, _dp]),
    "st_wrap_pbc_device": (_i32, [_vp, _dp, _i32, _i32, _i32, _vp, _i64, _i64, _vp]),
    "st_atom_extents_device": (_i32, [_vp, _i32, _dp, _dp, _dp, _vp, _i64, _i64, _dp]),
    "st_xyz_header": (_i32, [ctypes.c_char_p, ctypes.POINTER(StXyzInfo)]),
    "st_parse_xyz_device": (_i32, [_vp, _vp, _i64, _i64, _i32, _vp, _i64, _vp, ctypes.POINTER(_i32),
                                   ctypes.c_char_p, _i32, ctypes.POINTER(_i64), _vp]),
    "st_read_xyz": (_i32, [_vp, ctypes.c_char_p, ctypes.POINTER(StXyzInfo), _dp, _i64, ctypes.POINTER(_i32),
                           ctypes.POINTER(_i32), ctypes.c_char_p, _i32]),
    "st_fortran_parse_real": (_i32, [ctypes.c_char_p, _i64, _dp, ctypes.POINTER(_i32)]),
    "st_d2bi_set_lattice": (_i32, [_vp, _i32]),
    "st_d2bi_set_supercell_tilt1a": (_i32, [_vp, _vp, _d, ctypes.c_char_p, _d, _d, _vp, _i64, _i64,
                                            ctypes.POINTER(StTiltInfo)]),
    "st_find_best_rotation": (_i32, [_vp, _d, _dp, _dp, _i32, ctypes.POINTER(_i32), ctypes.c_char_p, _d, _d, _d,
                                     _dp, _dp, ctypes.POINTER(StTiltInfo)]),
    "st_tilt_scores": (_i32, [_vp, _d, _dp, _i32, _dp, _dp, _i32, _d, _dp]),
    "st_tilt_screen": (_i32, [_vp, _d, _dp, _i32, _dp, _dp, _i32, _d, _dp, _dp]),
    "st_tilt_to_dark_field": (_i32, [_d, _dp, ctypes.POINTER(_i32), _d, _d, _d, _d, _dp, _dp, _dp]),
    "st_read_extinction_distances": (_i32, [ctypes.c_char_p, _i32, ctypes.POINTER(_i32), _i32, _dp,
                                            ctypes.POINTER(_i32)]),
    "st_permitted_reflections": (_i32, [_i32, _d, ctypes.POINTER(_i32), _i32, ctypes.POINTER(_i32)]),
    "st_rotmat_to_quaternion": (_i32, [_dp, _dp]),
    "st_quaternion_to_rotmat": (_i32, [_dp, _dp]),
    "st_slerp": (_i32, [_dp, _dp, _d, _dp]),
}

_lib = None


def lib():
    """The loaded libstem.so (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libstem.so is not built: run `python -c \"import __graft_entry__ as g; g.build()\"` "
                               "or `python simulated_tem_gb300/build.py`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return sorted(_PROTOS)


def check(code, ctx=None):
    if code != ST_OK:
        msg = lib().st_last_error(ctx).decode() if ctx else ""
        raise StemError(code, msg)


def peaks_lib():
    if not os.path.exists(PEAKS_PATH):
        raise RuntimeError("libstem_peaks.so is not built")
    L = ctypes.CDLL(PEAKS_PATH)
    L.stp_measure_peaks.restype = _i32
    L.stp_measure_peaks.argtypes = [_dp]
    return L
