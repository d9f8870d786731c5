"""The LAMMPS data files d2bi reads, on the host side (no GPU): the header as
readHeader_lammps reads it, the exact number parser the GPU reader uses (against
Python's correctly rounded float()), and the oracle's atom-line reader against the
reference's own input (the first 3,000 atoms of Data/test/test.i111_loop_W.lammps)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import _lib, imaging

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
HEAD = os.path.join(GOLDEN, "w_loop_head.lammps")


def parse_real(s):
    out = ctypes.c_double()
    used = ctypes.c_int32()
    b = s.encode()
    code = _lib.lib().st_parse_real(b, len(b), ctypes.byref(out), ctypes.byref(used))
    return (out.value, used.value) if code == _lib.ST_OK else (None, 0)


def test_header_of_the_reference_input():
    info = imaging.lammps_header(HEAD)
    assert info.n_atoms == 3000 and info.n_types == 1
    assert list(info.lo) == [0.0, 0.0, 0.0] and list(info.hi) == [75.9648] * 3
    with open(HEAD, "rb") as f:
        text = f.read()
    assert text[info.data_offset:].startswith(b"1 1 0.7921030044820485 ")


def test_oracle_reader_matches_the_fixture_positions():
    info = imaging.lammps_header(HEAD)
    x, ty = O.read_lammps_atoms(HEAD, info.data_offset, info.n_atoms)
    want = np.load(os.path.join(GOLDEN, "w_loop_input.npz"))["pos"][:3000]
    assert np.array_equal(x, want) and (ty == 1).all()


def random_numbers(rng, n):
    out = []
    for i in range(n):
        k = i % 7
        v = float(rng.uniform(-1000, 1000))
        if k == 0:
            out.append(repr(v))
        elif k == 1:
            out.append("%.6f" % v)
        elif k == 2:
            out.append("%.17e" % v)
        elif k == 3:
            out.append(("%.15E" % v).replace("E", "D"))
        elif k == 4:  # long digit strings, beyond 19 significant digits
            digits = "".join(rng.choice(list("0123456789"), size=int(rng.integers(20, 40))))
            out.append("%s%s.%se%d" % ("-" if rng.random() < 0.5 else "", rng.integers(1, 9), digits,
                                       rng.integers(-15, 15)))
        elif k == 5:  # tiny and huge magnitudes
            out.append(repr(v * 10.0 ** int(rng.integers(-18, 30))))
        else:  # exact binary midpoints printed in full
            a = np.float64(rng.uniform(1, 2))
            b = np.nextafter(a, 3.0)
            from decimal import Decimal
            out.append(str((Decimal(float(a)) + Decimal(float(b))) / 2))
    return out


def test_number_parser_is_correctly_rounded():
    rng = np.random.default_rng(11)
    for s in random_numbers(rng, 20000):
        got, used = parse_real(s)
        want = float(s.replace("D", "e").replace("d", "e"))
        assert got is not None and used == len(s), s
        assert got == want and np.signbit(got) == np.signbit(want), s


@pytest.mark.parametrize("s,want,used", [
    ("0", 0.0, 1), ("-0.0", -0.0, 4), ("007", 7.0, 3), (".5", 0.5, 2), ("5.", 5.0, 2), ("1d3", 1000.0, 3),
    ("+2.5D-2", 0.025, 7), ("1.5 2", 1.5, 3), ("3,4", 3.0, 1)])
def test_number_parser_forms(s, want, used):
    got, u = parse_real(s)
    assert got == want and u == used and np.signbit(got) == np.signbit(want)


@pytest.mark.parametrize("s", ["", "+", "-", "e5", "abc", "1e", "1e+", "1e400", "1e-400"])
def test_number_parser_refuses(s):
    assert parse_real(s)[0] is None
