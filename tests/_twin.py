"""
Builds the same system twice -- once on the GPU path (taichimps_gb300), once on
the CPU oracle -- from one set of arrays, and compares them.
"""

from __future__ import annotations

import numpy as np

PAIR_STYLES = {
    "hooke": dict(style="hooke", kw=dict(kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5)),
    "hooke/history": dict(style="hooke/history", kw=dict(kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5)),
    "hertz": dict(style="hertz", kw=dict(kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5)),
    "hertz/history": dict(style="hertz/history", kw=dict(kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5)),
    "granular/mindlin": dict(style="granular", kw=dict(
        normal="hertz/material", normal_coeffs=[5e6, 0.5, 0.3], tangential="mindlin",
        tangential_coeffs=[None, 1.0, 0.5], damping="coeff_restitution")),
    "granular/linear_history": dict(style="granular", kw=dict(
        normal="hooke", normal_coeffs=[2e5, 30.0], tangential="linear_history", tangential_coeffs=[5e4, 0.5, 0.4],
        damping="mass_velocity")),
    "granular/nohistory": dict(style="granular", kw=dict(
        normal="hertz", normal_coeffs=[2e5, 10.0], tangential="linear_nohistory", tangential_coeffs=[0.5, 0.4],
        damping="viscoelastic")),
    "granular/tsuji": dict(style="granular", kw=dict(
        normal="hertz", normal_coeffs=[2e5, 0.7], tangential="mindlin", tangential_coeffs=[3e4, 1.0, 0.4],
        damping="tsuji", limit_damping=True)),
    "granular/velocity": dict(style="granular", kw=dict(
        normal="hooke", normal_coeffs=[2e5, 5.0], tangential="none", damping="velocity")),
    # the triaxial configuration's contact: hertz/material, coeff_restitution, mindlin, rolling EPSD
    "granular/rolling": dict(style="granular", kw=dict(
        normal="hertz/material", normal_coeffs=[5e6, 0.5, 0.3], tangential="mindlin",
        tangential_coeffs=[None, 1.0, 0.5], damping="coeff_restitution", rolling="epsd",
        rolling_coeffs=[1e3, 50.0, 0.1])),
}


def gpu_pair(name, dom, limit_damping=False):
    from taichimps_gb300.GRANULAR import GranHertz, GranHertzHistory, GranHooke, GranHookeHistory, PairGranular
    spec = PAIR_STYLES[name]
    kw = dict(spec["kw"])
    cls = {"hooke": GranHooke, "hooke/history": GranHookeHistory, "hertz": GranHertz,
           "hertz/history": GranHertzHistory}.get(spec["style"])
    if cls is not None:
        return cls(domain=dom, limit_damping=limit_damping, **kw)
    return PairGranular(domain=dom, **kw)


def oracle_pair(O, name, limit_damping=False):
    spec = PAIR_STYLES[name]
    kw = dict(spec["kw"])
    if spec["style"] != "granular":
        kw["limit_damping"] = limit_damping
    return O.OraclePair(spec["style"], **kw)


def dense_packing(rng, n, box, radius_lo, radius_hi, jitter=0.02):
    """Jittered simple-cubic points with radii wide enough to overlap (many contacts)."""
    side = int(np.ceil(n ** (1.0 / 3.0)))
    sp = box / side
    g = (np.arange(side) + 0.5) * sp
    pts = np.array([[a, b, c] for a in g for b in g for c in g])[:n]
    pts = pts + rng.uniform(-jitter * sp, jitter * sp, size=pts.shape)
    rad = rng.uniform(radius_lo, radius_hi, size=n)
    return pts % box, rad


def make_twin(O, x, radius, density, box_lo, box_hi, boundary=("p", "p", "p"), v=None, w=None, skin=0.1,
              pair="hooke/history", dt=1e-4, max_nb=32, cundall=None, deform=None, nve=True, tag=None):
    import taichimps_gb300 as G

    n = len(x)
    dom = G.Domain(boxlo=box_lo, boxhi=box_hi, boundary=boundary)
    atom = G.AtomSystem(max_atoms=n)
    atom.add_particles(x=x, radius=radius, density=density, v=v, omega=w, tag=tag)
    nl = G.NeighborList(domain=dom, skin=skin, max_atoms=n, max_neighbors_per_atom=max_nb)
    hist = G.ContactHistory(max_atoms=n, max_neighbors=max_nb)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=gpu_pair(pair, dom), dt=dt)
    if nve:
        sim.add_fix(G.FixNVESphere(domain=dom))
    if cundall is not None:
        sim.add_fix(G.FixDampingCundall(domain=dom, gamma_lin=cundall[0], gamma_ang=cundall[1]))
    if deform is not None:
        sim.add_fix(G.FixDeformPressure(domain=dom, **deform))

    odom = O.OracleDomain.make(box_lo, box_hi, boundary)
    oat = O.OracleAtoms(x=x, radius=radius, density=density, v=v, omega=w, tag=tag)
    onl = O.OracleNeighbor(odom, skin=skin, max_neighbors=max_nb)
    ohist = O.OracleHistory(max_nb)
    fixes = []
    if cundall is not None:
        fixes.append(O.OracleCundall(*cundall))
    if deform is not None:
        fixes.append(O.OracleDeform(odom, **deform))
    osim = O.OracleSim(odom, oat, onl, ohist, oracle_pair(O, pair), dt, fixes=fixes)
    if not nve:
        class _NoNVE:
            def initial_integrate(self, a, d):
                pass

            def final_integrate(self, a, d):
                pass
        osim.integrator = _NoNVE()
    return sim, osim


def rel_err(a, b):
    """max |a - b| / max |b| (0 when both vanish)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.abs(b).max() if b.size else 0.0
    d = np.abs(a - b).max() if b.size else 0.0
    return 0.0 if s == 0.0 and d == 0.0 else d / (s if s > 0 else 1.0)


def gpu_state(sim):
    a = sim.atom
    n = a.nlocal
    return {"x": a.x.to_numpy()[:n], "v": a.v.to_numpy()[:n], "omega": a.omega.to_numpy()[:n],
            "f": a.f.to_numpy()[:n], "torque": a.torque.to_numpy()[:n], "virial": a.virial.to_numpy()[:n]}


def oracle_state(osim):
    a = osim.atoms
    return {"x": a.x, "v": a.v, "omega": a.omega, "f": a.f, "torque": a.torque, "virial": a.virial}
