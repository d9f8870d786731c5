"""The .xyz reader on the GPU (st_read_xyz, st_parse_xyz_device) against the oracle's
input0: every column bit for bit, species numbers in order of first appearance, the
6-character names, bad lines, the species limit, and columns beyond ldx."""
import ctypes

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import _lib, imaging, synth

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


def _write(tmp_path, n_species=3, cells=(8, 8, 6), seed=2, extra=2, form="lattice", name="c.xyz"):
    cell = synth.small_cell(cells, seed=seed)
    rng = np.random.default_rng(seed)
    pool = ["Fe", "W", "Chromium", "Vanadium", "Ta"] if n_species <= 5 else ["X%d" % k for k in range(n_species)]
    sp = rng.choice(pool[:n_species], size=len(cell.pos))
    ex = None if extra == 0 else rng.normal(size=(len(cell.pos), extra))
    p = str(tmp_path / name)
    synth.write_xyz(p, cell.pos, cell.a_super, species=sp, extra=ex, form=form)
    return p, cell


@pytest.mark.parametrize("form", ["lattice", "boxsize", "header"])
def test_read_matches_oracle(ctx, tmp_path, form):
    p, cell = _write(tmp_path, form=form)
    x, types, species, info = ctx.read_xyz(p)
    xo, to, so = O.read_xyz_atoms(p, O.xyz_header(p))
    assert np.array_equal(x, xo)
    assert np.array_equal(x[:, :3], cell.pos)
    assert np.array_equal(types, to) and species == so


def test_columns_and_leading_dimension(ctx, tmp_path):
    p, cell = _write(tmp_path, extra=2)  # 5 columns
    info = imaging.xyz_header(p)
    n = info.n_read
    for ldx in (3, 5, 14):
        x = np.full((n, ldx), -7.0)
        t = np.zeros(n, dtype=np.int32)
        ns = ctypes.c_int32()
        ctx._check(imaging.lib().st_read_xyz(ctx.handle, p.encode(), ctypes.byref(info), imaging._ptr(x), ldx,
                                             t.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(ns),
                                             None, 0))
        xo, _, _ = O.read_xyz_atoms(p, O.xyz_header(p), ldx=5)
        k = min(ldx, 5)
        assert np.array_equal(x[:, :k], xo[:, :k])
        assert np.all(x[:, k:] == -7.0)  # rows beyond the file's columns are left alone
        assert ns.value == 3


def test_many_species_first_appearance(ctx, tmp_path):
    p, _ = _write(tmp_path, n_species=300, cells=(20, 20, 12))
    x, types, species, _ = ctx.read_xyz(p)
    xo, to, so = O.read_xyz_atoms(p, O.xyz_header(p))
    assert np.array_equal(types, to) and species == so and len(species) == 300


def test_too_many_species(ctx, tmp_path):
    cell = synth.small_cell((10, 10, 6), seed=1)
    n = len(cell.pos)
    assert n > 1001
    sp = ["S%04d" % (k % 1001) for k in range(n)]
    p = str(tmp_path / "many.xyz")
    synth.write_xyz(p, cell.pos, cell.a_super, species=sp)
    with pytest.raises(_lib.StemError):
        ctx.read_xyz(p)


def test_bad_line_reported(ctx, tmp_path):
    p, cell = _write(tmp_path, extra=0)
    with open(p) as f:
        lines = f.read().splitlines()
    lines[2 + 57] = "Fe 1.0 2.0"  # the 58th atom line misses a number
    with open(p, "w") as f:
        f.write("\n".join(lines) + "\n")
    info = imaging.xyz_header(p)
    with open(p, "rb") as f:
        f.seek(info.data_offset)
        text = np.frombuffer(f.read(), dtype=np.uint8)
    d_t = torch.from_numpy(text.copy()).cuda()
    d_x = torch.zeros((info.n_read, 3), dtype=torch.float64, device="cuda")
    bad, _ = ctx.parse_xyz_device(d_t.data_ptr(), len(text), info.n_read, 3, d_x.data_ptr(), 3)
    assert bad == 57


def test_unaligned_device_text(ctx, tmp_path):
    p, cell = _write(tmp_path, extra=1)
    info = imaging.xyz_header(p)
    with open(p, "rb") as f:
        f.seek(info.data_offset)
        text = np.frombuffer(f.read(), dtype=np.uint8)
    buf = torch.zeros(len(text) + 3, dtype=torch.uint8, device="cuda")
    buf[3:] = torch.from_numpy(text.copy()).cuda()
    d_x = torch.zeros((info.n_read, 4), dtype=torch.float64, device="cuda")
    d_t = torch.zeros(info.n_read, dtype=torch.int32, device="cuda")
    bad, species = ctx.parse_xyz_device(buf.data_ptr() + 3, len(text), info.n_read, 4, d_x.data_ptr(), 4,
                                        d_t.data_ptr())
    assert bad == -1
    xo, to, so = O.read_xyz_atoms(p, O.xyz_header(p))
    assert np.array_equal(d_x.cpu().numpy(), xo) and np.array_equal(d_t.cpu().numpy(), to) and species == so
