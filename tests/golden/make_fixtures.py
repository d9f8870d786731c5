"""Regenerate the golden fixtures in this folder from the reference's own data.

Reads, as text or image bytes only, the reference repository's shipped test
data and writes compact fixtures beside this script:

* ``w_loop_input.npz``   -- the 27,847-atom W input of the ``testD2BI`` ctest
  (``Data/test/test.i111_loop_W.lammps``): positions in file order and box.
* ``w_loop_dat.npz``     -- the shipped 94x94 dark-field image and its header
  (``Data/test/test.i111_loop_W.lammps.g2_0_0.k0.00_0.00_1.00_ng1.00.dat``).
* ``w_loop_png.npz``     -- the 16-bit greyscale levels of the shipped PNG of
  that image (decoded here with zlib; no imaging library is needed).
* ``w_loop_dat_text.json`` -- the same .dat file as text: its header lines, the size
  line, and its first and last '(1000f12.7)' records (the output-format fixture).
* ``w_loop_head.lammps`` -- the first 3,000 atom lines of that input with its header
  (the atom count line set to 3000): the reader's fixture.
* ``w_xi_V200_T300.dat`` -- the extinction-distance table the ``testD2BI`` ctest reads
  with ``-xifile`` (``Data/ExtinctionDistances/extinctionDistances.W_V200_T300.dat``),
  copied line for line: the fixture of the ``-ng`` tilt search.
* ``linkcell_kat.json``  -- the 200 points and the stored neighbour list of
  ``test/testLib_LinkCell3D.f90``.
* ``electrons_kat.json`` -- the stored wavelength/velocity strings of
  ``test/testLib_RelativisticElectrons.f90``.
* ``quaternion_kat.json`` -- the rotation matrix of ``test/testLib_Quaternions.f90`` and
  its stored quaternion components (the test's first output line).
* ``golden_section_kat.json`` -- the brackets of ``test/testLib_GoldenSection.f90`` (each
  search must end at a local minimum of the test's function).
* ``tokenizer_kat.json`` -- the real-array string of ``test/testNBAX_StringTokenizers.f90``
  and its stored '(100g24.12)' output.

Usage: ``python tests/golden/make_fixtures.py /path/to/reference``.
"""
import json
import os
import re
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_lammps(path):
    with open(path) as f:
        lines = f.read().splitlines()
    box = np.zeros((3, 2))
    n_atoms = None
    start = None
    for i, line in enumerate(lines):
        for k, tag in enumerate(("xlo", "ylo", "zlo")):
            if tag in line:
                lo, hi = line.split()[:2]
                box[k] = float(lo), float(hi)
        if line.strip().endswith("atoms") and n_atoms is None:
            n_atoms = int(line.split()[0])
        if line.startswith("Atoms"):
            start = i + 2
            break
    pos = np.empty((n_atoms, 3))
    ids = np.empty(n_atoms, dtype=np.int64)
    for j in range(n_atoms):
        tok = lines[start + j].split()
        ids[j] = int(tok[0])
        pos[j] = [float(t) for t in tok[2:5]]
    return box, ids, pos


def read_dat(path):
    with open(path) as f:
        lines = f.read().splitlines()
    header = {}
    body_start = None
    for i, line in enumerate(lines):
        if line.startswith("#"):
            key, _, rest = line[1:].strip().partition("  ")
            header[key.strip()] = [float(v) for v in rest.split()] if not key.startswith("d2bi") else rest
        else:
            nx, ny = (int(v) for v in line.split())
            body_start = i + 1
            break
    vals = np.array([float(v) for line in lines[body_start:] for v in line.split()])
    assert vals.size == nx * ny
    img = vals.reshape(ny, nx).T.copy()  # column-major (x fastest) in the file
    return header, img


def decode_png16(path):
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos = 8
    idat = b""
    width = height = None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8]
        chunk = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if ctype == b"IHDR":
            width, height, depth, colour, _, _, interlace = struct.unpack(">IIBBBBB", chunk)
            assert depth == 16 and colour == 0 and interlace == 0
        elif ctype == b"IDAT":
            idat += chunk
        elif ctype == b"IEND":
            break
    raw = zlib.decompress(idat)
    bpp, stride = 2, 2 * width
    out = np.zeros((height, stride), dtype=np.int64)
    prev = np.zeros(stride, dtype=np.int64)
    p = 0
    for y in range(height):
        ftype = raw[p]
        row = np.frombuffer(raw[p + 1:p + 1 + stride], dtype=np.uint8).astype(np.int64)
        p += 1 + stride
        cur = np.zeros(stride, dtype=np.int64)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ftype == 0:
                pred = 0
            elif ftype == 1:
                pred = a
            elif ftype == 2:
                pred = b
            elif ftype == 3:
                pred = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[x] = (row[x] + pred) & 0xFF
        out[y] = cur
        prev = cur
    levels = (out[:, 0::2] << 8) | out[:, 1::2]
    return levels.astype(np.uint16)  # [row y, column x]


def lammps_head(path, n=3000):
    with open(path) as f:
        lines = f.read().split("\n")
    k = next(i for i, line in enumerate(lines) if line.startswith("Atoms")) + 2
    head = [("%d atoms" % n) if line.strip().endswith(" atoms") else line for line in lines[:k]]
    return "\n".join(head + lines[k:k + n]) + "\n"


def dat_text(path):
    with open(path) as f:
        lines = f.read().split("\n")
    k = next(i for i, line in enumerate(lines) if not line.startswith("#"))
    records = [line for line in lines[k + 1:] if line]
    return {"header_lines": lines[:k + 1], "n_records": len(records), "first_record": records[0],
            "last_record": records[-1]}


def linkcell_kat(path):
    with open(path) as f:
        text = f.read()
    body = text[text.index("xx = reshape("):]
    body = body[:body.index("/),(/ 3,200 /)")]
    nums = [float(v.replace("d0", "")) for v in re.findall(r"-?\d+\.\d+d0", body)]
    pts = np.array(nums).reshape(200, 3)
    neigh = []
    for m in re.finditer(r'"neigh\s+(\d+) id\s+(\d+) dx\s+(-?[\d.]+)\s+(-?[\d.]+)\s+(-?[\d.]+) \|dx\|\s+([\d.]+)', text):
        neigh.append({"n": int(m.group(1)), "id": int(m.group(2)),
                      "dx": [float(m.group(k)) for k in (3, 4, 5)], "absdx": float(m.group(6))})
    m = re.search(r'" max storage per cell\s+(\d+)', text)
    max_storage = int(m.group(1))
    m = re.search(r'"atom 100 at\s+(-?[\d.]+)\s+(-?[\d.]+)\s+(-?[\d.]+)', text)
    atom100 = [float(m.group(k)) for k in (1, 2, 3)]
    return {"points": pts.tolist(), "cells": [6, 4, 5], "cutoff": 1.0, "atom100": atom100,
            "neighbours": neigh, "max_count": max_storage}


def electrons_kat(path):
    with open(path) as f:
        text = f.read()
    wl = float(re.search(r'"wavelength\s+([\d.]+)', text).group(1))
    v = float(re.search(r'"velocity\s+([\d.]+)', text).group(1))
    volts = float(re.search(r'"accelerating voltage V =\s+([\d.]+)', text).group(1))
    return {"V": volts, "wavelength": wl, "velocity": v}


def quaternion_kat(path):
    with open(path) as f:
        text = f.read()
    body = text[text.index("R1(1:3,1:3) = reshape("):]
    body = body[:body.index("(/3,3/)")]
    r1 = [float(v.replace("d0", "")) for v in re.findall(r"-?\d+\.\d+d0", body)]
    out = re.search(r'output0 = \(/\s*"([^"]*)"', text).group(1).split()
    return {"R1_column_major": r1, "q_wxyz": out}


def golden_section_kat(path):
    with open(path) as f:
        text = f.read()
    pairs = re.findall(r"x1 = (-?[\d.]+)d0 ; x3 = (-?[\d.]+)d0", text)
    ok = int(re.search(r"passcount==(\d+)", text).group(1))
    return {"brackets": [[float(a), float(b)] for a, b in pairs], "pass_count": ok}


def tokenizer_kat(path):
    with open(path) as f:
        text = f.read()
    src = re.search(r"dummy = '([-0-9.de ]+)'\s*\n\s*output\(10\)", text).group(1)
    lines = re.findall(r'"(\s+1\.00000000000\s+[^"]*)"', text)
    return {"string": src, "g24_12": lines[0].split()}


def main(ref):
    box, ids, pos = read_lammps(os.path.join(ref, "Data/test/test.i111_loop_W.lammps"))
    np.savez_compressed(os.path.join(HERE, "w_loop_input.npz"), box=box, ids=ids, pos=pos)
    dat = "Data/test/test.i111_loop_W.lammps.g2_0_0.k0.00_0.00_1.00_ng1.00"
    header, img = read_dat(os.path.join(ref, dat + ".dat"))
    np.savez_compressed(os.path.join(HERE, "w_loop_dat.npz"), img=img,
                        header=json.dumps(header))
    with open(os.path.join(HERE, "w_loop_head.lammps"), "w") as f:
        f.write(lammps_head(os.path.join(ref, "Data/test/test.i111_loop_W.lammps")))
    with open(os.path.join(HERE, "w_loop_dat_text.json"), "w") as f:
        json.dump(dat_text(os.path.join(ref, dat + ".dat")), f)
    with open(os.path.join(ref, "Data/ExtinctionDistances/extinctionDistances.W_V200_T300.dat")) as f:
        xi_table = f.read()
    with open(os.path.join(HERE, "w_xi_V200_T300.dat"), "w") as f:
        f.write(xi_table)
    levels = decode_png16(os.path.join(ref, dat + ".png"))
    np.savez_compressed(os.path.join(HERE, "w_loop_png.npz"), levels=levels)
    with open(os.path.join(HERE, "linkcell_kat.json"), "w") as f:
        json.dump(linkcell_kat(os.path.join(ref, "test/testLib_LinkCell3D.f90")), f, indent=1)
    with open(os.path.join(HERE, "electrons_kat.json"), "w") as f:
        json.dump(electrons_kat(os.path.join(ref, "test/testLib_RelativisticElectrons.f90")), f, indent=1)
    with open(os.path.join(HERE, "quaternion_kat.json"), "w") as f:
        json.dump(quaternion_kat(os.path.join(ref, "test/testLib_Quaternions.f90")), f, indent=1)
    with open(os.path.join(HERE, "golden_section_kat.json"), "w") as f:
        json.dump(golden_section_kat(os.path.join(ref, "test/testLib_GoldenSection.f90")), f, indent=1)
    with open(os.path.join(HERE, "tokenizer_kat.json"), "w") as f:
        json.dump(tokenizer_kat(os.path.join(ref, "test/testNBAX_StringTokenizers.f90")), f, indent=1)
    print("wrote fixtures:", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of the reference checkout>")
    main(sys.argv[1])
