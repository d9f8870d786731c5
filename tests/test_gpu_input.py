"""The LAMMPS atom lines parsed on the GPU: the reference's own input (its first 3,000
atoms), blocks in every number form and separator a list-directed read accepts, against
Python's correctly rounded float() and the oracle's reader, and the first bad line of
malformed blocks."""
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import imaging, synth

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
HEAD = os.path.join(GOLDEN, "w_loop_head.lammps")


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


def parse_block(ctx, text, n_atoms):
    b = np.frombuffer(text.encode(), dtype=np.uint8)
    d_t = torch.from_numpy(b.copy()).cuda() if b.size else torch.zeros(1, dtype=torch.uint8, device="cuda")
    d_x = torch.zeros((max(n_atoms, 1), 3), dtype=torch.float64, device="cuda")
    d_ty = torch.zeros(max(n_atoms, 1), dtype=torch.int32, device="cuda")
    bad = ctx.parse_atoms_device(d_t.data_ptr(), b.size, n_atoms, d_x.data_ptr(), d_ty.data_ptr(),
                                 stream=torch.cuda.current_stream().cuda_stream)
    return bad, d_x.cpu().numpy()[:n_atoms], d_ty.cpu().numpy()[:n_atoms]


def test_reads_the_reference_input(ctx):
    x, ty, info = ctx.read_lammps(HEAD)
    want = np.load(os.path.join(GOLDEN, "w_loop_input.npz"))["pos"][:3000]
    assert np.array_equal(x, want) and (ty == 1).all()
    xo, _ = O.read_lammps_atoms(HEAD, info.data_offset, info.n_atoms)
    assert np.array_equal(x, xo)


def test_number_forms_and_separators(ctx):
    rng = np.random.default_rng(3)
    n = 20000
    vals = rng.uniform(-800, 800, size=(n, 3))
    lines, want = [], np.zeros((n, 3))
    forms = [lambda v: repr(float(v)), lambda v: "%.6f" % v, lambda v: "%.17e" % v,
             lambda v: ("%.15E" % v).replace("E", "D"), lambda v: "%+.10g" % v, lambda v: "%.3f" % v]
    seps = [" ", "\t", "  ", " , ", ","]
    for i in range(n):
        toks = [forms[(i + k) % len(forms)](vals[i, k]) for k in range(3)]
        want[i] = [float(t.replace("D", "e")) for t in toks]
        sep = seps[i % len(seps)]
        tail = ["", " 0 0 0", "\t1 -1 2", " extra words"][i % 4]
        end = "\r\n" if i % 9 == 0 else "\n"
        lines.append(("  " if i % 5 == 0 else "") + sep.join([str(i + 1), str(1 + i % 3)] + toks) + tail + end)
    bad, x, ty = parse_block(ctx, "".join(lines), n)
    assert bad == -1
    assert np.array_equal(x, want)
    assert np.array_equal(ty, 1 + np.arange(n) % 3)


def test_unaligned_text_buffer(ctx):
    """A text block starting at an odd device address (inside a larger buffer)."""
    text = "".join("%d 2 %r %r %r\n" % (i + 1, 0.25 * i, -1.5, 1e-3 * i) for i in range(5000))
    b = np.frombuffer(("x" + text).encode(), dtype=np.uint8)
    d_t = torch.from_numpy(b.copy()).cuda()
    d_x = torch.zeros((5000, 3), dtype=torch.float64, device="cuda")
    bad = ctx.parse_atoms_device(d_t.data_ptr() + 1, b.size - 1, 5000, d_x.data_ptr(),
                                 stream=torch.cuda.current_stream().cuda_stream)
    assert bad == -1
    want = np.array([[0.25 * i, -1.5, 1e-3 * i] for i in range(5000)])
    assert np.array_equal(d_x.cpu().numpy(), want)


def test_bad_lines_are_reported(ctx):
    good = "".join("%d 1 %r %r %r\n" % (i + 1, 0.5 * i, 1.0, 2.0) for i in range(100))
    lines = good.split("\n")
    for k, broken in ((37, "38 1 0.5 1.0"), (5, "6 1 0.5 abc 2.0"), (64, ""), (0, "1 1 1.0e 2 3")):
        bl = list(lines)
        bl[k] = broken
        assert parse_block(ctx, "\n".join(bl), 100)[0] == k
    assert parse_block(ctx, good, 120)[0] == 100  # fewer lines than atoms


def test_large_file_matches_oracle(ctx, tmp_path):
    cell = synth.make_cell(40, 40, 30, synth.BASE_SEED + 9, n_voids=3, void_radius=(5.0, 9.0), with_screw=True)
    path = str(tmp_path / "cell.lammps")
    synth.write_lammps(path, cell.pos, np.diag(cell.a_super))
    x, ty, info = ctx.read_lammps(path)
    assert info.n_atoms == len(cell.pos)
    assert np.array_equal(x, cell.pos)  # shortest round-trip strings read back exactly
    xo, _ = O.read_lammps_atoms(path, info.data_offset, info.n_atoms)
    assert np.array_equal(x, xo)
