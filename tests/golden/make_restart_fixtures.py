"""
Golden LAMMPS restart files written by the reference's own writer
(src/taichimps/restart.py write_restart), for tests/test_cpu_restart.py.

The reference's restart module needs only numpy and the standard library, so
it runs in this container although the rest of the reference (Taichi) does
not; it is loaded straight from its file.  Its writer reads the system
through a few attributes (atom fields with .to_numpy(), the domain's box and
periodicity, the history's touching_by_atom, the pair's submodels), which are
provided here over seeded arrays.  Outputs, beside this script:

  restart_inputs.npz        the arrays the files were written from
  restart_granular.bin      pair granular (hertz/material, mindlin, coeff_restitution) + contact history
  restart_history_only.bin  no force field, contact history
  restart_plain.bin         no force field, no history

Run:  python tests/golden/make_restart_fixtures.py <reference root>
"""

from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def load_reference_restart(root: Path):
    spec = importlib.util.spec_from_file_location("reference_restart", root / "src" / "taichimps" / "restart.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["reference_restart"] = mod
    spec.loader.exec_module(mod)
    return mod


class _Field:
    def __init__(self, a):
        self.a = a

    def to_numpy(self):
        return self.a


class _Atom:
    def __init__(self, d):
        self.nlocal = len(d["radius"])
        self.x, self.v, self.omega = _Field(d["x"]), _Field(d["v"]), _Field(d["omega"])
        self.radius, self.rmass = _Field(d["radius"]), _Field(d["rmass"])
        self.tag, self.atom_type = _Field(d["tag"]), _Field(d["atom_type"])


class _Domain:
    def __init__(self, d):
        self.periodicity = d["periodicity"]
        self.triclinic = False
        self.boxlo, self.boxhi = d["boxlo"], d["boxhi"]
        self.tilt = [0.0, 0.0, 0.0]


class _History:
    """touching_by_atom: each contact once, under its lower-index atom, in that atom's sense."""

    def __init__(self, d):
        self.own = [[] for _ in range(len(d["radius"]))]
        for i, j, s in zip(d["c_i"], d["c_j"], d["c_shear"]):
            self.own[int(i)].append((int(d["tag"][j]), np.array(s)))

    def touching_by_atom(self, nlist, n):
        return self.own


class _Pair:
    submodels = {"normal": ("hertz/material", [5.0e6, 0.5, 0.3]), "damping": ("coeff_restitution", []),
                 "tangential": ("mindlin", [-1.0, 1.0, 0.5]), "rolling": ("none", []),
                 "twisting": ("none", []), "heat": ("none", [])}
    limit_damping = 0


def inputs(seed: int = 20261204, n: int = 40) -> dict:
    rng = np.random.default_rng(seed)
    boxlo = np.array([-1.5, 0.25, 2.0])
    boxhi = boxlo + np.array([9.0, 8.5, 10.25])
    d = {
        "x": boxlo + rng.random((n, 3)) * (boxhi - boxlo),
        "v": rng.normal(0.0, 0.3, (n, 3)),
        "omega": rng.normal(0.0, 1.5, (n, 3)),
        "radius": rng.uniform(0.4, 0.6, n),
        "tag": (rng.permutation(n) * 3 + 7).astype(np.int32),   # unordered, gapped tags
        "atom_type": rng.integers(1, 3, n).astype(np.int32),
        "boxlo": boxlo, "boxhi": boxhi, "periodicity": np.array([1, 1, 0], dtype=np.int32),
        "timestep": np.int64(123456789012), "dt": np.float64(3.5e-5),
    }
    d["rmass"] = (4.0 / 3.0) * np.pi * d["radius"] ** 3 * rng.uniform(2.0, 3.0, n)
    # contacts: random pairs i < j, each once, at most 5 per atom
    pairs, deg = set(), np.zeros(n, dtype=int)
    while len(pairs) < 70:
        i, j = sorted(rng.choice(n, 2, replace=False))
        if (i, j) not in pairs and deg[i] < 5 and deg[j] < 5:
            pairs.add((int(i), int(j)))
            deg[i] += 1
            deg[j] += 1
    pairs = sorted(pairs, key=lambda p: (p[0], rng.random()))  # an atom's partners in no particular order
    d["c_i"] = np.array([p[0] for p in pairs], dtype=np.int64)
    d["c_j"] = np.array([p[1] for p in pairs], dtype=np.int64)
    d["c_shear"] = rng.normal(0.0, 1e-3, (len(pairs), 3))
    return d


def main(root: str) -> None:
    ref = load_reference_restart(Path(root))
    d = inputs()
    np.savez(HERE / "restart_inputs.npz", **d)
    atom, dom = _Atom(d), _Domain(d)
    step, dt = int(d["timestep"]), float(d["dt"])
    ref.write_restart(HERE / "restart_granular.bin", atom, dom, timestep=step, dt=dt, history=_History(d),
                      pair=_Pair(), nlist=object())
    ref.write_restart(HERE / "restart_history_only.bin", atom, dom, timestep=step, dt=dt, history=_History(d),
                      pair=None, nlist=object())
    ref.write_restart(HERE / "restart_plain.bin", atom, dom, timestep=step, dt=dt)
    for f in ("restart_granular.bin", "restart_history_only.bin", "restart_plain.bin"):
        print(f, (HERE / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
