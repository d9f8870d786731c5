"""The .xyz files d2bi reads, on the host side (no GPU): the header as readHeader and
getSupercell0 read it (src/Lib_XYZFiles.f90:507-626, 905-1058), with the reference's own
string tools (NBAX_StringTokenizers.f90) pinned to its unit test, and the oracle's atom
reader (input0, :756-892) against the positions written."""
import json
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import imaging, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fortran_g(x, d=12):
    """Fortran G24.12 editing for the values of the tokenizer test."""
    if x == 0:
        return "0." + "0" * (d - 1)
    e = int(np.floor(np.log10(abs(x)))) + 1
    if 0 <= e <= d:
        return "%.*f" % (d - e, x)
    m = "%.*e" % (d - 1, x)  # d.ddd e+xx -> 0.dddd E+xx+1
    mant, ex = m.split("e")
    digits = mant.replace("-", "").replace(".", "")
    return "%s0.%sE%+03d" % ("-" if x < 0 else "", digits, int(ex) + 1)


def test_tokenizer_kat():
    """test/testNBAX_StringTokenizers.f90: ParseRealArray of its string, '(100g24.12)'."""
    with open(os.path.join(GOLDEN, "tokenizer_kat.json")) as f:
        k = json.load(f)
    toks = k["string"].split()
    got_o = [fortran_g(O.fortran_parse_real(t)) for t in toks]
    got_p = [fortran_g(imaging.fortran_parse_real(t)) for t in toks]
    assert got_o == k["g24_12"] and got_p == k["g24_12"]


@pytest.mark.parametrize("s", ["1.0d0", "-2.0e-2", "123456", "-0.0", "123456789.987654321", "28.7", ".5", "-.25e+3",
                               "5.", "1e5", "7.25D-3", "0.1", "3.14159265358979", "1-2", "12.5abc", "  42", "e",
                               "-", "1.2.3", "0.000000000000000000001", "99999999999999999999999999999999999.5"])
def test_parse_real_product_equals_oracle(s):
    """ParseReal is not correctly rounded (digits times powers of 0.1, then 10 ** e); the
    product's header reader and the oracle restate it to the same bits."""
    a, b = imaging.fortran_parse_real(s), O.fortran_parse_real(s)
    assert (a is None and b is None) or (a == b or (np.isnan(a) and np.isnan(b)))


def test_parse_real_is_the_reference_arithmetic():
    # -2.0e-2 = 2 * (1 / 10**2); 0.3 = 3 * 0.1 (not the nearest double of 0.3)
    assert imaging.fortran_parse_real("-2.0e-2") == -(2.0 * (1 / 100.0))
    assert imaging.fortran_parse_real("0.3") == 0.1 * 3
    assert imaging.fortran_parse_real("0.3") != 0.3
    assert imaging.fortran_parse_real("-0.0") == 0.0 and np.signbit(imaging.fortran_parse_real("-0.0")) == False


def _fields(h):
    out = {}
    for f, _ in h._fields_:
        v = getattr(h, f)
        out[f] = v if isinstance(v, (int, float, bytes)) else list(v)
    return out


@pytest.mark.parametrize("form", ["lattice", "boxsize", "header"])
@pytest.mark.parametrize("comments", [(), ("a comment", "% another")])
def test_header_matches_oracle(tmp_path, form, comments):
    cell = synth.small_cell((6, 5, 4), seed=3)
    a = np.array(cell.a_super) * np.array([1.0, 1.1, 0.97])  # not round numbers
    p = str(tmp_path / "c.xyz")
    synth.write_xyz(p, cell.pos, a, form=form, comments=comments,
                    extra=np.arange(2 * len(cell.pos), dtype=float).reshape(-1, 2))
    h, ho = imaging.xyz_header(p), O.xyz_header(p)
    assert _fields(h) == _fields(ho)
    assert h.n_atoms == h.n_read == len(cell.pos) and h.n_columns == 5 and h.supercell_ok == 1
    assert h.supercell_kind == {"lattice": 1, "boxsize": 2, "header": 3}[form]
    got = np.array(list(h.a_super)).reshape(3, 3).T
    ref = np.array([[imaging.fortran_parse_real(repr(float(v))) for v in row] for row in a])
    assert np.array_equal(got if form != "boxsize" else np.diag(np.diag(got)),
                          ref if form != "boxsize" else np.diag(np.diag(ref)))


def test_header_edge_cases(tmp_path):
    p = str(tmp_path / "e.xyz")
    # nine Lattice values then more numbers on the line: the first nine; a "super cell"
    # comment with repeats scales the vectors; a CRLF file
    with open(p, "w") as f:
        f.write('3\nLattice="2 0 0 0 3 0 0 0 4" energy=-1.5 pbc="T T T"\nW 0 0 0\nW 1 1 1\nW 1.5 0.5 2\n')
    h = imaging.xyz_header(p)
    assert _fields(h) == _fields(O.xyz_header(p))
    assert list(h.a_super) == [2.0, 0, 0, 0, 3.0, 0, 0, 0, 4.0] and h.supercell_ok
    with open(p, "w", newline="") as f:
        f.write("! super cell 2 2 1\r\n# 1.0 0.0 0.0\r\n# 0.0 1.5 0.0\r\n# 0.0 0.0 2.0\r\n2 atoms\r\ndesc\r\n"
                "Fe 0.1 0.2 0.3\r\nFe 0.4 0.5 0.6\r\n")
    h = imaging.xyz_header(p)
    assert _fields(h) == _fields(O.xyz_header(p))
    assert h.supercell_kind == 3 and list(h.repeats) == [2, 2, 1]
    assert list(h.a_super) == [2.0, 0.0, 0.0, 0.0, 3.0, 0.0, 0.0, 0.0, 2.0]
    assert h.n_header_lines == 4 and h.n_atoms == 2
    # the count line "12.5": parseInt gives 12, the list-directed read fails
    with open(p, "w") as f:
        f.write("12.5\nboxsize 1 2 3\nFe 0 0 0\n")
    h = imaging.xyz_header(p)
    assert (h.n_atoms, h.n_read) == (12, -1) and _fields(h) == _fields(O.xyz_header(p))
    # a LAMMPS file is flagged; fewer than three numbers on the first atom line is an error
    with open(p, "w") as f:
        f.write("LAMMPS data\n\n3 atoms\n")
    assert imaging.xyz_header(p).lammps == 1
    with open(p, "w") as f:
        f.write("1\nboxsize 1 1 1\nFe 0.0 1.0\n")
    with pytest.raises(Exception):
        imaging.xyz_header(p)
    with pytest.raises(Exception):
        imaging.xyz_header(str(tmp_path / "missing.xyz"))


def test_oracle_reader_reads_the_written_positions(tmp_path):
    cell = synth.small_cell((5, 5, 4), seed=9)
    rng = np.random.default_rng(4)
    sp = rng.choice(["Fe", "Chromium", "W"], size=len(cell.pos))
    p = str(tmp_path / "r.xyz")
    synth.write_xyz(p, cell.pos, cell.a_super, species=sp)
    x, types, names = O.read_xyz_atoms(p, O.xyz_header(p))
    assert np.array_equal(x, cell.pos)
    # character(len=6) keeps six characters; numbers follow the order of first appearance
    order = list(dict.fromkeys(s[:6].ljust(6) for s in sp))
    assert names == order
    assert np.array_equal(types, [order.index(s[:6].ljust(6)) + 1 for s in sp])
