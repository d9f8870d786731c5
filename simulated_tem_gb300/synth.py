"""Seeded synthetic bcc cells for the imaging workloads.

There is no network and no dataset: every workload is a seeded synthetic bcc
Fe cell (a0 = 2.87 A) built here with numpy's PCG64.  Sites a0 (i, j, k) and
a0 (i + 1/2, j + 1/2, k + 1/2), Gaussian jitter per coordinate, optional
straight screw dislocation along z through the cell centre
(u_z = b atan2(y - y0, x - x0) / 2 pi, applied after the jitter so no atom sits
on the line), and spherical voids removed with the minimum-image distance.
Workload k uses seed 20261203 + k; its sub-streams come from
``SeedSequence.spawn`` in the order jitter, void centres, void radii, extra.
"""
import dataclasses

import numpy as np

A0_FE = 2.87
BASE_SEED = 20261203


def bcc_sites(nx, ny, nz, a0=A0_FE):
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    corner = np.stack([i, j, k], axis=-1).reshape(-1, 3).astype(np.float64)
    pos = np.concatenate([corner, corner + 0.5], axis=0) * a0
    return pos


def streams(seed, n=4):
    ss = np.random.SeedSequence(seed)
    return [np.random.Generator(np.random.PCG64(s)) for s in ss.spawn(n)]


def remove_voids(pos, box, centres, radii):
    keep = np.ones(len(pos), dtype=bool)
    for c, r in zip(centres, radii):
        d = pos - c
        d -= box * np.round(d / box)  # minimum image
        keep &= (d * d).sum(axis=1) > r * r
    return pos[keep]


def screw(pos, box, b=A0_FE):
    x0, y0 = box[0] / 2, box[1] / 2
    out = pos.copy()
    out[:, 2] += b * np.arctan2(pos[:, 1] - y0, pos[:, 0] - x0) / (2 * np.pi)
    return out


@dataclasses.dataclass
class Cell:
    """A periodic cell: supercell matrix (columns) and positions (N, 3)."""
    a_super: np.ndarray
    pos: np.ndarray
    name: str = ""

    @property
    def n_atoms(self):
        return len(self.pos)


def make_cell(nx, ny, nz, seed, n_voids=0, void_radius=(10.0, 10.0), jitter=0.05, with_screw=False, a0=A0_FE,
              name=""):
    rj, rc, rr, _ = streams(seed)
    box = np.array([nx, ny, nz], dtype=np.float64) * a0
    pos = bcc_sites(nx, ny, nz, a0)
    pos = pos + rj.normal(0.0, jitter, size=pos.shape)
    if with_screw:
        pos = screw(pos, box, b=a0)
    if n_voids:
        centres = rc.uniform(0.0, 1.0, size=(n_voids, 3)) * box
        radii = rr.uniform(void_radius[0], void_radius[1], size=n_voids)
        pos = remove_voids(pos, box, centres, radii)
    return Cell(np.diag(box), np.ascontiguousarray(pos), name)


def void_cell_128k():
    """40 x 40 x 40 cells (128,000 sites), 8 voids of radius 10 A, jitter 0.05 A."""
    return make_cell(40, 40, 40, BASE_SEED + 1, n_voids=8, void_radius=(10.0, 10.0), name="bcc Fe 40^3, 8 voids")


def screw_cell_1p2m():
    """100 x 100 x 60 cells (1.2M sites), screw dislocation along z, 20 voids of radius U(5, 15) A."""
    return make_cell(100, 100, 60, BASE_SEED + 2, n_voids=20, void_radius=(5.0, 15.0), with_screw=True,
                     name="bcc Fe 100x100x60, screw + 20 voids")


def small_cell(n=(8, 8, 6), seed=7, n_voids=1, radius=(4.0, 6.0), with_screw=True):
    """A few-thousand-atom cell for parity tests."""
    return make_cell(n[0], n[1], n[2], seed, n_voids=n_voids, void_radius=radius, with_screw=with_screw,
                     name="small bcc Fe")


def uneven_cells(count=256, seed=BASE_SEED + 4, lo=10_000, hi=500_000):
    """Independent bcc cells with atom counts log-uniform in [lo, hi], aspect ratios U(0.5, 2),
    Poisson(10) voids of radius U(4, 20) A and s_g ~ U(-0.02, 0.02) per cell (as (cell, s_g) pairs)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n_target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        ax, ay = rng.uniform(0.5, 2.0, size=2)
        # nx ny nz * 2 = n_target with nx : ny : nz = ax : ay : 1
        nz = max(2, int(round((n_target / 2 / (ax * ay)) ** (1.0 / 3.0))))
        nx, ny = max(2, int(round(ax * nz))), max(2, int(round(ay * nz)))
        nv = int(rng.poisson(10))
        sg = float(rng.uniform(-0.02, 0.02))
        cell = make_cell(nx, ny, nz, int(rng.integers(1 << 31)), n_voids=nv, void_radius=(4.0, 20.0),
                         name="cell %d" % i)
        out.append((cell, sg))
    return out


def write_lammps(path, pos, box_hi, mass=55.845, box_lo=(0.0, 0.0, 0.0)):
    """A LAMMPS data file in the layout of LAMMPS' write_data (atom_style atomic, one type):
    the reference's input format (src/Lib_XYZFiles.f90:628-716, 1061-1117).  Coordinates are
    written as the shortest decimal strings that read back to the same doubles."""
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    head = ["LAMMPS data file written by simulated_tem_gb300.synth", "", "%d atoms" % n, "1 atom types", ""]
    for k, ax in enumerate("xyz"):
        head.append("%r %r %slo %shi" % (float(box_lo[k]), float(box_hi[k]), ax, ax))
    head += ["", "Masses", "", "1 %r" % mass, "", "Atoms # atomic", ""]
    with open(path, "w") as f:
        f.write("\n".join(head) + "\n")
        chunk = 100_000
        for s in range(0, n, chunk):
            p = pos[s:s + chunk]
            f.write("".join("%d 1 %r %r %r 0 0 0\n" % (s + i + 1, a, b, c)
                            for i, (a, b, c) in enumerate(p.tolist())))


def write_xyz(path, pos, a_super, species=None, extra=None, form="lattice", comments=()):
    """An .xyz file the reference reads (src/Lib_XYZFiles.f90:507-626, 756-892): optional
    comment lines, the atom count, a description line carrying the supercell, then one line
    per atom: species, x, y, z and any extra columns.  form: "lattice" (extended xyz,
    Lattice="..." with the nine components of the cell vectors), "boxsize" (PARCAS, the
    three box lengths) or "header" (a "supercell" comment line with 1 1 1 repeats and the
    three cell vectors, one per line).  Coordinates are written as the shortest decimal
    strings that read back to the same doubles."""
    pos = np.asarray(pos, dtype=np.float64)
    a = np.asarray(a_super, dtype=np.float64)
    n = len(pos)
    species = ["Fe"] * n if species is None else list(species)
    lines = ["# " + c for c in comments]
    if form == "header":
        lines.append("# supercell 1 1 1")
        for k in range(3):
            lines.append("# " + " ".join(repr(float(v)) for v in a[:, k]))
        desc = "positions in Angstrom"
    elif form == "boxsize":
        desc = "boxsize %r %r %r" % (float(a[0, 0]), float(a[1, 1]), float(a[2, 2]))
    else:
        desc = 'Lattice="%s" Properties=species:S:1:pos:R:3' % " ".join(repr(float(v)) for v in a.T.reshape(-1))
    lines += ["%d" % n, desc]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
        chunk = 100_000
        for s in range(0, n, chunk):
            rows = []
            for i in range(s, min(n, s + chunk)):
                vals = [repr(float(v)) for v in pos[i]]
                if extra is not None:
                    vals += [repr(float(v)) for v in np.atleast_1d(extra[i])]
                rows.append("%s %s\n" % (species[i], " ".join(vals)))
            f.write("".join(rows))
