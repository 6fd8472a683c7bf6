"""
LAMMPS ``atom_style sphere`` data files: read (as the reference's
src/taichimps/data_reader.py:30-142 does) and write.

Atoms lines are ``id type diameter density x y z``; Velocities lines are
``id vx vy vz wx wy wz``.  radius = diameter / 2.  Written files use 17
significant digits so every double round-trips exactly.
"""

from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np


@dataclass
class LAMMPSData:
    natoms: int
    natom_types: int
    boxlo: list
    boxhi: list
    tilt: list
    x: np.ndarray
    radius: np.ndarray
    density: np.ndarray
    v: np.ndarray
    omega: np.ndarray
    tag: np.ndarray
    atom_type: np.ndarray


def read_data(filepath) -> LAMMPSData:
    path = Path(filepath)
    if not path.exists():
        raise FileNotFoundError(f"Data file not found: {path}")
    natoms, ntypes = 0, 1
    lo, hi, tilt = [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.0, 0.0, 0.0]
    sections: dict[str, list[str]] = {"header": []}
    cur = "header"
    with open(path, "r", encoding="utf-8", errors="ignore") as fh:
        for line in fh:
            s = line.split("#")[0].strip()
            if not s:
                continue
            low = s.lower()
            if low.startswith("atoms"):
                cur = "atoms"
                sections[cur] = []
                continue
            if low.startswith("velocities"):
                cur = "velocities"
                sections[cur] = []
                continue
            sections[cur].append(s)
    for s in sections["header"]:
        t = s.split()
        if len(t) >= 2 and t[1] == "atoms":
            natoms = int(t[0])
        elif len(t) >= 3 and t[1] == "atom" and t[2] == "types":
            ntypes = int(t[0])
        elif len(t) >= 4 and t[2:4] in (["xlo", "xhi"], ["ylo", "yhi"], ["zlo", "zhi"]):
            k = "xyz".index(t[2][0])
            lo[k], hi[k] = float(t[0]), float(t[1])
        elif len(t) >= 6 and t[3:6] == ["xy", "xz", "yz"]:
            tilt = [float(v) for v in t[0:3]]
    rows = sections.get("atoms", [])
    n = len(rows)
    tags = np.zeros(n, dtype=np.int32)
    types = np.zeros(n, dtype=np.int32)
    rad = np.zeros(n)
    dens = np.zeros(n)
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    w = np.zeros((n, 3))
    where = {}
    for i, s in enumerate(rows):
        t = s.split()
        tags[i], types[i] = int(t[0]), int(t[1])
        rad[i] = 0.5 * float(t[2])
        dens[i] = float(t[3])
        x[i] = [float(t[4]), float(t[5]), float(t[6])]
        where[int(t[0])] = i
    for s in sections.get("velocities", []):
        t = s.split()
        i = where.get(int(t[0]))
        if i is None:
            continue
        v[i] = [float(t[1]), float(t[2]), float(t[3])]
        if len(t) >= 7:
            w[i] = [float(t[4]), float(t[5]), float(t[6])]
    return LAMMPSData(n, ntypes, lo, hi, tilt, x, rad, dens, v, w, tags, types)


def write_data(filepath, boxlo, boxhi, x, radius, density, v=None, omega=None, tag=None,
               atom_type=None, title: str = "taichimps_gb300 data file") -> None:
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    rad = np.broadcast_to(np.asarray(radius, dtype=np.float64), (n,))
    dens = np.broadcast_to(np.asarray(density, dtype=np.float64), (n,))
    tag = np.arange(1, n + 1) if tag is None else np.asarray(tag)
    types = np.ones(n, dtype=np.int32) if atom_type is None else np.asarray(atom_type)
    with open(filepath, "w") as fh:
        fh.write(f"{title}\n\n{n} atoms\n{int(types.max()) if n else 1} atom types\n\n")
        for k, ax in enumerate("xyz"):
            fh.write(f"{boxlo[k]:.17g} {boxhi[k]:.17g} {ax}lo {ax}hi\n")
        fh.write("\nAtoms # sphere\n\n")
        for i in range(n):
            fh.write(f"{int(tag[i])} {int(types[i])} {2.0 * rad[i]:.17g} {dens[i]:.17g} "
                     f"{x[i, 0]:.17g} {x[i, 1]:.17g} {x[i, 2]:.17g}\n")
        if v is not None or omega is not None:
            vv = np.zeros((n, 3)) if v is None else np.asarray(v)
            ww = np.zeros((n, 3)) if omega is None else np.asarray(omega)
            fh.write("\nVelocities\n\n")
            for i in range(n):
                fh.write(f"{int(tag[i])} {vv[i, 0]:.17g} {vv[i, 1]:.17g} {vv[i, 2]:.17g} "
                         f"{ww[i, 0]:.17g} {ww[i, 1]:.17g} {ww[i, 2]:.17g}\n")
