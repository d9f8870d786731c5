"""The C-ABI library loads on a machine without a GPU and exports every entry
point that include/*.h declares (no compute calls here)."""
import glob
import os
import re

from simulated_tem_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(st_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_the_boundary():
    names = declared_functions()
    for required in ("st_create", "st_destroy", "st_last_error", "st_image", "st_image_device", "st_blur",
                     "st_blur_device", "st_get_stats"):
        assert required in names


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in sorted(declared_functions()) if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding covers every declaration
    assert set(_lib.exported_symbols()) >= declared_functions()


def test_host_mirror_runs_without_gpu():
    """The host-side set-up needs no device."""
    import numpy as np
    from simulated_tem_gb300 import imaging, synth
    cell = synth.small_cell((6, 6, 5), seed=2)
    t, x, ap = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.01)
    G, aa = t.image_geometry(len(x), n_prec=3)
    assert G.Mx > 0 and len(aa) == 3 and np.isfinite(aa).all()


def test_errors_without_context():
    import ctypes
    L = _lib.lib()
    assert L.st_image(None, None, None, 3, 0, None, 1, 0, None) == _lib.ST_ERR_ARG
    assert L.st_blur(None, None, 1, 1, 1.0, None) == _lib.ST_ERR_ARG
    h = ctypes.c_void_p()
    assert L.st_d2bi_create(ctypes.byref(h), None, 1, 1, 1, 1.0, None, None, 200.0, 4, 4) == _lib.ST_ERR_ARG


def test_tuning_variants_are_named_without_gpu():
    """st_tune_variants / st_tune_variant_name are host-only: six slab-ring variants, the
    tile shape and slab capacity in each name, "invalid" out of range."""
    L = _lib.lib()
    n = L.st_tune_variants()
    assert n == 6
    names = [L.st_tune_variant_name(v).decode() for v in range(n)]
    assert names == ["8x4 slab128", "8x4 slab96", "4x8 slab128", "4x8 slab96", "16x2 slab128", "16x2 slab96"]
    assert L.st_tune_variant_name(-1).decode() == "invalid" and L.st_tune_variant_name(n).decode() == "invalid"
