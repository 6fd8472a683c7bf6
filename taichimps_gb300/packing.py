"""
Seeded packings of polydisperse spheres in a periodic cube.

Random sequential insertion stalls near solid fraction 0.38, below the 0.40 and
0.45 the benchmark configurations ask for, so packings are made this way:

1. diameters drawn uniform in [dmin, dmax] (numpy PCG64, fixed seed);
2. the cube edge L set so that sum(pi d^3 / 6) / L^3 equals the target fraction;
3. centres placed on randomly chosen sites of the smallest FCC lattice with at
   least n sites, each jittered by up to `jitter` of the lattice constant
   (0.5 % by default: at solid fraction 0.45 the FCC nearest-neighbour
   distance is only just above the largest diameter);
4. remaining overlaps removed by repeatedly pushing each overlapping pair apart
   along its line of centres (periodic minimum image) until none is left.

The result has no overlapping pair, so it starts with no contacts.
"""

from __future__ import annotations

import math

import numpy as np


def _fcc_sites(m: int) -> np.ndarray:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3)
    return (g[:, None, :] + base[None, :, :]).reshape(-1, 3)


def remove_overlaps(x: np.ndarray, radius: np.ndarray, L, max_iter: int = 500, margin: float = 1e-9,
                    relist: int = 0):
    """Push overlapping pairs apart until none overlaps (periodic box of edge L, a scalar or three edges).

    Candidate pairs are found once (within 2 r_max plus a slack larger than
    the total displacement the pushes may add); later passes only look at
    pairs with an atom that moved in the previous pass.  If the pushes moved
    an atom beyond the slack, the candidate list is rebuilt and the removal
    continues from there, up to `relist` times (else it raises).
    """
    for attempt in range(relist + 1):
        try:
            return _remove_overlaps_once(x, radius, L, max_iter, margin)
        except _BeyondSlack as e:
            if attempt == relist:
                raise RuntimeError("overlap removal moved atoms beyond the candidate-pair slack") from None
            x = e.x


class _BeyondSlack(Exception):
    def __init__(self, x):
        super().__init__("beyond slack")
        self.x = x


def _remove_overlaps_once(x, radius, L, max_iter, margin):
    from scipy.spatial import cKDTree

    x = np.mod(x, L)
    rmax = float(radius.max())
    slack = 0.25 * rmax
    pairs = cKDTree(x, boxsize=L).query_pairs(r=2.0 * rmax + slack, output_type="ndarray")
    if len(pairs) == 0:
        return x
    pi, pj = pairs[:, 0], pairs[:, 1]
    need_all = radius[pi] + radius[pj] + margin
    x0 = x.copy()
    active = np.ones(len(pi), dtype=bool)
    for _ in range(max_iter):
        i, j, need = pi[active], pj[active], need_all[active]
        d = x[i] - x[j]
        d -= L * np.round(d / L)
        r = np.sqrt((d * d).sum(1))
        bad = r < need
        if not bad.any():
            disp = x - x0
            disp -= L * np.round(disp / L)
            if np.sqrt((disp * disp).sum(1)).max() >= 0.5 * slack:
                raise _BeyondSlack(x)
            return x
        i, j, d, r, need = i[bad], j[bad], d[bad], r[bad], need[bad]
        r = np.maximum(r, 1e-12)
        push = (0.5 * (need - r) * 1.05 + margin)[:, None] * (d / r[:, None])
        delta = np.zeros_like(x)
        np.add.at(delta, i, push)
        np.add.at(delta, j, -push)
        x = np.mod(x + delta, L)
        moved = np.zeros(len(x), dtype=bool)
        moved[i] = True
        moved[j] = True
        active = moved[pi] | moved[pj]
    raise RuntimeError("overlap removal did not converge")


def make_packing(n: int, dmin: float, dmax: float, phi: float, seed: int, jitter: float = 0.005,
                 vel_sigma: float = 0.0):
    """Returns dict(x, radius, L, v) for n spheres at solid fraction phi."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(dmin, dmax, size=n)
    L = float((np.sum(math.pi / 6.0 * d ** 3) / phi) ** (1.0 / 3.0))
    m = int(math.ceil((n / 4.0) ** (1.0 / 3.0)))
    while 4 * m ** 3 < n:
        m += 1
    sites = _fcc_sites(m)
    pick = rng.choice(len(sites), size=n, replace=False)
    a = L / m
    x = (sites[pick] + 0.25) * a + rng.uniform(-jitter, jitter, size=(n, 3)) * a
    radius = 0.5 * d
    x = remove_overlaps(x, radius, L, relist=20)
    v = rng.normal(0.0, vel_sigma, size=(n, 3)) if vel_sigma > 0.0 else np.zeros((n, 3))
    return {"x": x, "radius": radius, "L": L, "v": v}


def _fcc_sites_box(mx: int, my: int, mz: int) -> np.ndarray:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(mx), np.arange(my), np.arange(mz), indexing="ij"), -1).reshape(-1, 3)
    return (g[:, None, :] + base[None, :, :]).reshape(-1, 3)


def make_packing_box(n: int, dmin: float, dmax: float, phi: float, seed: int, jitter: float = 0.005,
                     vel_sigma: float = 0.0):
    """make_packing for any n: at solid fraction 0.45 with d up to 1.2 the FCC nearest-neighbour distance is
    only just above the largest diameter, so the lattice must be nearly full.  The periodic box is shaped to
    an FCC lattice of mx x my x mz cells (edges within 4:3 of each other) with the fewest sites >= n, at the
    same solid fraction.  Returns dict(x, radius, L (three edges), v)."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(dmin, dmax, size=n)
    vol = float(np.sum(math.pi / 6.0 * d ** 3) / phi)
    m0 = (n / 4.0) ** (1.0 / 3.0)
    lo, hi = max(1, int(math.floor(0.7 * m0))), int(math.ceil(1.4 * m0)) + 1
    best = None
    for mx in range(lo, hi + 1):
        for my in range(mx, hi + 1):
            for mz in range(my, hi + 1):
                sites = 4 * mx * my * mz
                if sites < n or 3 * mz > 4 * mx:
                    continue
                if best is None or sites < best[0]:
                    best = (sites, mx, my, mz)
    _, mx, my, mz = best
    a = (vol / (mx * my * mz)) ** (1.0 / 3.0)
    L = a * np.array([mx, my, mz], dtype=np.float64)
    sites = _fcc_sites_box(mx, my, mz)
    pick = rng.choice(len(sites), size=n, replace=False)
    x = (sites[pick] + 0.25) * a + rng.uniform(-jitter, jitter, size=(n, 3)) * a
    radius = 0.5 * d
    x = remove_overlaps(x, radius, L, relist=20)
    v = rng.normal(0.0, vel_sigma, size=(n, 3)) if vel_sigma > 0.0 else np.zeros((n, 3))
    return {"x": x, "radius": radius, "L": L, "v": v}


def config1(seed: int = 1, n: int = 4000):
    """4,000 spheres, d ~ U[0.9, 1.1], phi 0.40, v ~ N(0, 0.1^2), rho 2.5."""
    p = make_packing(n, 0.9, 1.1, 0.40, seed, jitter=0.05, vel_sigma=0.1)
    p["density"] = 2.5
    return p


def config2(seed: int = 2, n: int = 1_000_000):
    """1,000,000 spheres, d ~ U[0.8, 1.2], phi 0.45, at rest, rho 2.5."""
    p = make_packing(n, 0.8, 1.2, 0.45, seed)
    p["density"] = 2.5
    return p


def compress_packing(n: int, seed: int, dmin: float = 0.8, dmax: float = 1.2, density: float = 2.5,
                     kn: float = 1.0e5, xmu: float = 0.5, ptarget: float = 1.0, pgain: float = 1.0,
                     max_rate: float = 0.005, cycles: int = 100, relax_cycles: int = 10, cycle_steps: int = 2000,
                     dt: float = 5e-4, precision: str = "fp64", phi0: float = 0.3, jitter: float = 0.3):
    """An isotropically compressed packing: `make_packing_box` at solid
    fraction `phi0` with the sites jittered by `jitter` lattice constants (a
    disordered gas; sites on an unjittered lattice would jam as a crystal of
    the largest spheres), then gran/hertz/history (kn, kt = 2/7 kn, gamman 50,
    gammat 25, xmu) with Cundall damping 0.7 and deform/pressure on x/y/z
    (target `ptarget`, couple xyz, remap x).  The run is cut into cycles of
    `cycle_steps` steps that each start at rest: Hertz collisions are nearly
    elastic and Cundall damping does not slow a free sphere, so without the
    quench the servo would stop on the kinetic pressure of a granular gas.
    `cycles` at `max_rate`, then `relax_cycles` at a tenth of it.  The rate
    is kept well below (equilibrium overlap) / (diameter x contact time) --
    about 0.01 at kn 1e5 and p 1 -- or the contacts overshoot and the servo
    stops on dynamic pressure.  Returns
    positions wrapped into the final box, radii, box edges and lower corner,
    the last pressure tensor and the solid fraction.  Runs on the GPU path."""
    from . import (AtomSystem, ContactHistory, Domain, FixDampingCundall, FixDeformPressure, FixNVESphere,
                   GranHertzHistory, NeighborList, Simulation)

    p = make_packing_box(n, dmin, dmax, phi0, seed, jitter=jitter)
    L0 = [float(v) for v in p["L"]]
    state = {"x": p["x"], "lo": [0.0] * 3, "hi": L0}
    tensor = np.zeros(6)
    for c in range(cycles + relax_cycles):
        rate = max_rate if c < cycles else 0.1 * max_rate
        dom = Domain(boxlo=state["lo"], boxhi=state["hi"], boundary=("p", "p", "p"))
        atom = AtomSystem(max_atoms=n)
        atom.add_particles(x=state["x"], radius=p["radius"], density=density)
        nl = NeighborList(domain=dom, skin=0.1, max_atoms=n, max_neighbors_per_atom=32)
        hist = ContactHistory(max_atoms=n, max_neighbors=32)
        pair = GranHertzHistory(domain=dom, kn=kn, kt=kn * 2.0 / 7.0, gamman=50.0, gammat=25.0, xmu=xmu,
                                dampflag=1)
        sim = Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=dt, precision=precision)
        sim.add_fix(FixNVESphere(domain=dom))
        sim.add_fix(FixDampingCundall(domain=dom, gamma_lin=0.7, gamma_ang=0.7))
        fx = FixDeformPressure(domain=dom, axes={d: {"style": "pressure", "ptarget": ptarget, "pgain": pgain}
                                                for d in "xyz"}, couple="xyz", max_rate=rate, remap="x")
        sim.add_fix(fx)
        fx.record_pressure(4)
        sim.run(cycle_steps)
        tensor = fx.pressure_history([sim.timestep])[0]
        dom.pull()
        lo = np.array(dom.boxlo, dtype=np.float64)
        prd = np.array(dom.boxhi, dtype=np.float64) - lo
        x = atom.x.to_numpy()
        state = {"x": lo + np.mod(x - lo, prd), "lo": [float(a) for a in lo], "hi": [float(a) for a in lo + prd]}
    lo, hi = np.array(state["lo"]), np.array(state["hi"])
    vol_s = float(np.sum((4.0 / 3.0) * np.pi * p["radius"] ** 3))
    return {"x": state["x"], "radius": p["radius"], "lo": lo, "L": hi - lo, "pressure": tensor,
            "phi": vol_s / float(np.prod(hi - lo)), "density": density}


def tile_packing(cell: dict, reps=(4, 4, 4)) -> dict:
    """A periodic packing repeated reps[0] x reps[1] x reps[2] times in a box that many cells wide.

    A packing in a periodic box is also a packing of any whole number of
    copies of that box: every sphere keeps the neighbours it had through the
    cell's periodic images, so the tiled system starts with the cell's contact
    network (and pressure) in every copy.  Copies are laid out x fastest, then
    y, then z; positions are cell positions (wrapped into the cell) plus the
    copy's offset.  Returns dict(x, radius, lo, L, density, phi)."""
    lo = np.asarray(cell["lo"], dtype=np.float64)
    L = np.asarray(cell["L"], dtype=np.float64)
    x = lo + np.mod(np.asarray(cell["x"], dtype=np.float64) - lo, L)
    r = np.asarray(cell["radius"], dtype=np.float64)
    xs, rs = [], []
    for kz in range(reps[2]):
        for ky in range(reps[1]):
            for kx in range(reps[0]):
                xs.append(x + L * np.array([kx, ky, kz], dtype=np.float64))
                rs.append(r)
    Lt = L * np.array(reps, dtype=np.float64)
    out = {"x": np.concatenate(xs), "radius": np.concatenate(rs), "lo": lo.copy(), "L": Lt,
           "density": float(cell.get("density", 2.5))}
    out["phi"] = float(np.sum((4.0 / 3.0) * np.pi * out["radius"] ** 3) / np.prod(Lt))
    return out


# The contact-dense counterpart of the 1M-sphere servo run: a 15,625-sphere
# cell compressed to p = 1 with the run's own contact law, tiled 4 x 4 x 4.
DENSE_CELL_FILE = "dense_cell_hertz2e5_15625.npz"
DENSE_CELL_ARGS = dict(n=15625, seed=11, kn=2.0e5, dt=2.5e-4, max_rate=0.005, cycles=100, relax_cycles=40,
                       cycle_steps=2000, precision="mixed")


def dense_cell(path=None, regenerate: bool = False) -> dict:
    """The compressed cell of the dense 1M-sphere workload: gran/hertz/history kn 2e5 (kt 2/7 kn, gamman
    50, gammat 25, xmu 0.5), d ~ U[0.8, 1.2], density 2.5, 15,625 spheres compressed by compress_packing
    with DENSE_CELL_ARGS.  Read from the package's data file (written by this function on a GPU run with
    regenerate=True, so every run of the workload starts from the same bits)."""
    from pathlib import Path
    f = Path(path) if path is not None else Path(__file__).resolve().parent / "data" / DENSE_CELL_FILE
    if f.exists() and not regenerate:
        z = np.load(f)
        return {"x": z["x"], "radius": z["radius"], "lo": z["lo"], "L": z["L"], "pressure": z["pressure"],
                "phi": float(z["phi"]), "density": float(z["density"])}
    a = dict(DENSE_CELL_ARGS)
    cell = compress_packing(a.pop("n"), **a)
    f.parent.mkdir(parents=True, exist_ok=True)
    np.savez(f, x=cell["x"], radius=cell["radius"], lo=cell["lo"], L=cell["L"], pressure=cell["pressure"],
             phi=cell["phi"], density=cell["density"])
    return cell


def dense_config2(reps=(4, 4, 4), path=None) -> dict:
    """The dense workload's packing: the compressed cell tiled `reps` times (4 x 4 x 4 = 1,000,000
    spheres), at rest; dict(x, radius, L (three edges), lo, v, density, phi)."""
    t = tile_packing(dense_cell(path), reps)
    t["v"] = np.zeros_like(t["x"])
    return t
