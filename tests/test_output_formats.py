"""d2bi's output files on the host side (no GPU): the .dat header in Fortran editing and
the 16-bit PNG container, against the reference's shipped .dat and PNG files
(Data/test/*.dat, *.png, as fixtures in tests/golden/), and the oracle's restatements of
the '(1000f12.7)' records and the header."""
import json
import os
import sys
import zlib

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import imaging

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_fixtures as MF  # noqa: E402  (the PNG decoder of the fixtures)


def dat_text():
    with open(os.path.join(GOLDEN, "w_loop_dat_text.json")) as f:
        return json.load(f)


def header_fields(lines):
    """The .dat header's fields as d2bi wrote them (the values of the shipped file)."""
    rot = [float(v) for v in lines[10].split()[2:]]
    return dict(version="1.1.6", k=(0, 0, 1), g=(2, 0, 0), modg=3.97017, M=(4, 4), V=200.0, xi0=113.88929,
                xig=308.24709, ng=1.0, sg=0.00745, xmax=(74.731, 74.731, 74.881), aperpx=0.79502,
                rotation=np.array(rot))


def test_dat_header_reproduces_the_reference_file():
    d = dat_text()
    h = header_fields(d["header_lines"])
    assert imaging.format_dat_header(h, 94, 94).split("\n")[:-1] == d["header_lines"]
    ho = dict(h, rotation=list(h["rotation"]))
    assert O.dat_header(ho, 94, 94).split("\n")[:-1] == d["header_lines"]


def test_dat_header_fortran_editing():
    """Negative numbers, numbers too wide for the field (asterisks), zero decimals,
    4-index vectors and no n_g line: the library and the oracle agree."""
    h = dict(version="2.0", k=(-1, 0, 1, 0), g=(1, -1, 0, 0), modg=123456.789, M=(8, 8), V=1234567890.0,
             xi0=-0.0000049, xig=99999.999999, sg=-0.012345, xmax=(-1.0, 12345678.9, 0.0005), aperpx=0.5,
             rotation=np.array([-0.9999996, 0.0, 1e-9, -1e-9, 1.0, 0.5, 2.0, -2.0, 10000.0]), miller4=True)
    got = imaging.format_dat_header(h, 5, 123456789)
    want = O.dat_header(dict(h, rotation=list(h["rotation"])), 5, 123456789)
    assert got == want
    lines = got.split("\n")
    assert "# V (keV) **********" in lines  # 1234567890. needs 11 characters
    assert lines[1] == "# k           -1.000     0.000     1.000     0.000"
    assert lines[-2] == "       5********"


def test_oracle_records_reproduce_the_reference_file():
    """The oracle's F12.7 records equal the shipped file's first and last record when fed
    the values read back from them (pins the oracle's formatter)."""
    d = dat_text()
    for rec in (d["first_record"], d["last_record"]):
        vals = np.array([float(t) for t in rec.split()])
        assert O.format_f12_7(vals) == (rec + "\n").encode()
    assert d["n_records"] == (94 * 94 + 999) // 1000


def test_png_container_round_trip():
    """The shipped PNG's levels re-encoded by the library decode to the same pixels; the
    chunks carry valid CRCs and the zlib stream is valid."""
    lv = np.load(os.path.join(GOLDEN, "w_loop_png.npz"))["levels"]
    png = imaging.encode_png16(lv)
    assert png[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(png):
        n = int.from_bytes(png[pos:pos + 4], "big")
        ctype, data = png[pos + 4:pos + 8], png[pos + 8:pos + 8 + n]
        crc = int.from_bytes(png[pos + 8 + n:pos + 12 + n], "big")
        assert crc == zlib.crc32(ctype + data) & 0xFFFFFFFF
        chunks.append(ctype)
        if ctype == b"IDAT":
            raw = zlib.decompress(data)
            assert len(raw) == lv.shape[0] * (1 + 2 * lv.shape[1])
        pos += 12 + n
    assert chunks == [b"IHDR", b"IDAT", b"IEND"]
    path = os.path.join(GOLDEN, "..", "_png_round_trip.png")
    try:
        with open(path, "wb") as f:
            f.write(png)
        assert np.array_equal(MF.decode_png16(path), lv)
    finally:
        os.remove(path)


@pytest.mark.parametrize("shape", [(1, 1), (3, 40000), (700, 97)])
def test_png_container_block_boundaries(shape):
    """Images whose scanlines span several 65,535-byte stored blocks, and a 1 x 1 image."""
    rng = np.random.default_rng(sum(shape))
    lv = rng.integers(0, 65536, size=shape, dtype=np.uint16)
    png = imaging.encode_png16(lv)
    n = int.from_bytes(png[33:37], "big")
    raw = zlib.decompress(png[41:41 + n])
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(shape[0], 1 + 2 * shape[1])
    assert not rows[:, 0].any()
    got = (rows[:, 1::2].astype(np.uint16) << 8) | rows[:, 2::2]
    assert np.array_equal(got, lv)
