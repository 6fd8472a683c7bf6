"""
Whole steps through Simulation on the GPU vs the oracle's Simulation order:
trajectories, history carry-over across rebuilds, Cundall damping, the
pressure servo with remap x / remap v, and the reference's regression tests.
"""

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin, oracle_state, rel_err

pytestmark = pytest.mark.gpu


def test_config1_trajectory_100_steps(gpu, oracle):
    """4,000 spheres, gran/hooke/history, NVE (the reference's CPU config): 100 steps."""
    from taichimps_gb300.packing import config1
    p = config1(seed=1)
    L = p["L"]
    # compress the packing a little so contacts exist from step 0
    x = p["x"] * 0.93
    sim, osim = make_twin(oracle, x, p["radius"], 2.5, [0.0] * 3, [0.93 * L] * 3, v=p["v"],
                          pair="hooke/history", dt=1e-4, skin=0.1)
    sim.neighbor.every, sim.neighbor.delay = 1, 0
    sim.run(100)
    osim.run(100)
    g, o = gpu_state(sim), oracle_state(osim)
    assert np.abs(o["f"]).max() > 0
    assert sim.neighbor.build_count == osim.neighbor.build_count
    for k in ("x", "v", "omega"):
        assert rel_err(g[k], o[k]) < 1e-11, (k, rel_err(g[k], o[k]))
    for k in ("f", "torque"):
        assert rel_err(g[k], o[k]) < 1e-9, (k, rel_err(g[k], o[k]))


@pytest.mark.parametrize("pair", ["hertz/history", "granular/mindlin", "hooke", "granular/tsuji"])
def test_dense_steps_with_rebuilds(gpu, oracle, pair):
    """Dense overlapping packing, rebuild every step (check no): 30 steps."""
    rng = np.random.default_rng(11)
    x, r = dense_packing(rng, 512, 8.0, 0.5, 0.56)
    v = rng.normal(scale=0.05, size=x.shape)
    w = rng.normal(scale=0.5, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [8.0] * 3, v=v, w=w, pair=pair, dt=5e-5)
    sim.neighbor.check = False
    osim.neighbor.check = False
    sim.run(30)
    osim.run(30)
    g, o = gpu_state(sim), oracle_state(osim)
    assert sim.neighbor.build_count == osim.neighbor.build_count == 31
    for k in ("x", "v", "omega"):
        assert rel_err(g[k], o[k]) < 1e-11, (k, rel_err(g[k], o[k]))
    assert rel_err(g["f"], o["f"]) < 1e-9


def test_shear_history_survives_rebuild(gpu):
    """tests/test_lammps_parity.py:124-157 on the GPU: rebuild every step == never, rtol 1e-8."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(11)
    box = 6.0
    radius = 0.52 * (box / 4)
    side = 4
    sp = box / side
    pts = np.array([[(a + 0.5) * sp, (b + 0.5) * sp, (c + 0.5) * sp] for a in range(side) for b in range(side)
                    for c in range(side)])
    pts = (pts + rng.uniform(-0.02 * sp, 0.02 * sp, size=pts.shape)) % box
    vel = rng.normal(scale=0.05, size=pts.shape)
    omg = rng.normal(scale=0.5, size=pts.shape)

    def run(every):
        dom = G.Domain(boxlo=[0.0] * 3, boxhi=[box] * 3)
        atom = G.AtomSystem(max_atoms=64)
        atom.add_particles(x=pts, radius=radius, density=2650.0, v=vel, omega=omg)
        nl = G.NeighborList(domain=dom, max_atoms=64, max_neighbors_per_atom=32, skin=0.1)
        hist = G.ContactHistory(max_atoms=64, max_neighbors=32)
        pair = G.GranHookeHistory(domain=dom, kn=1.0e5, gamman=10.0, kt=5.0e4, gammat=5.0, xmu=0.5)
        sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=1e-4)
        sim.add_fix(G.FixNVESphere(domain=dom))
        if every:
            nl.check, nl.every = False, 1
        else:
            nl.check, nl.every = True, 10 ** 6
        sim.run(40)
        return atom.f.to_numpy()[:64].copy(), nl.build_count

    (f_re, b_re), (f_keep, b_keep) = run(True), run(False)
    assert b_re > b_keep
    scale = np.abs(f_keep).max()
    assert scale > 0.0
    np.testing.assert_allclose(f_re, f_keep, rtol=1e-8, atol=1e-8 * scale)


def test_cundall_and_servo_remap_x(gpu, oracle):
    """Config-2 step structure at small size: hertz/history + Cundall 0.7 + pressure servo
    (x/y/z, couple xyz, max/rate, remap x), 60 steps: box, pressure and state vs the oracle."""
    rng = np.random.default_rng(21)
    x, r = dense_packing(rng, 512, 8.2, 0.48, 0.56)
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap="x")
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [8.2] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7), deform=deform)
    sim.run(60)
    osim.run(60)
    sim.domain.pull()
    np.testing.assert_allclose(sim.domain.boxlo, osim.domain.boxlo, rtol=0, atol=1e-12)
    np.testing.assert_allclose(sim.domain.boxhi, osim.domain.boxhi, rtol=0, atol=1e-12)
    assert not np.allclose(osim.domain.prd, 8.2)
    g, o = gpu_state(sim), oracle_state(osim)
    for k in ("x", "v", "omega"):
        assert rel_err(g[k], o[k]) < 1e-11, (k, rel_err(g[k], o[k]))
    p_gpu = sim.fixes[-1].last_pressure()
    assert rel_err(p_gpu, osim.last_pressure) < 1e-10


@pytest.mark.parametrize("remap", ["v", "none"])
def test_servo_other_remaps(gpu, oracle, remap):
    rng = np.random.default_rng(22)
    x, r = dense_packing(rng, 343, 7.0, 0.5, 0.56)
    v = rng.normal(scale=0.1, size=x.shape)
    deform = dict(axes={"x": {"style": "pressure", "ptarget": 5.0, "pgain": 1e-2},
                        "y": {"style": "erate", "rate": -0.2}, "z": {"style": "pressure/mean", "ptarget": 5.0,
                                                                    "pgain": 1e-2}},
                  max_rate=0.5, remap=remap)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.0] * 3, v=v, pair="hooke/history", dt=1e-4,
                          deform=deform)
    sim.neighbor.check = False
    osim.neighbor.check = False
    sim.run(40)
    osim.run(40)
    sim.domain.pull()
    np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-13)
    g, o = gpu_state(sim), oracle_state(osim)
    for k in ("x", "v"):
        assert rel_err(g[k], o[k]) < 1e-11, (k, rel_err(g[k], o[k]))


def test_remap_x_moves_atoms_with_box(gpu):
    """tests/test_deform_remap_x.py:24-111 on the GPU path."""
    import taichimps_gb300 as G
    RADIUS, DENSITY, DT, ERATE = 5.0e-4, 2650.0, 1.0e-7, -0.05
    n_side = 6
    lo, hi = 0.0, n_side * 2.5 * RADIUS
    g = (np.arange(n_side) + 0.5) * (hi - lo) / n_side
    x = np.array([[a, b, c] for a in g for b in g for c in g])
    n = len(x)
    dom = G.Domain(boxlo=[lo] * 3, boxhi=[hi] * 3, boundary=("p", "p", "p"))
    atom = G.AtomSystem(max_atoms=n)
    atom.add_particles(x=x, radius=np.full(n, RADIUS), density=np.full(n, DENSITY))
    nlist = G.NeighborList(domain=dom, max_atoms=n, max_neighbors_per_atom=32, skin=0.4 * RADIUS)
    hist = G.ContactHistory(max_atoms=n, max_neighbors=32)
    pair = G.GranHertzHistory(domain=dom, kn=1e8, gamman=0.0, kt=1e8, gammat=0.0, xmu=0.3, dampflag=0)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nlist, history=hist, pair=pair, dt=DT)
    sim.add_fix(G.FixNVESphere(domain=dom))
    sim.add_fix(G.FixDeformPressure(domain=dom, nevery=1, remap="x", axes={"z": {"style": "erate", "rate": ERATE}}))
    sim.run(30)
    dom.pull()
    prd0 = np.full(3, hi - lo)
    prd = dom.boxhi - dom.boxlo
    assert prd[2] == pytest.approx(prd0[2] * (1.0 + ERATE * 30 * DT), rel=1e-9)
    assert prd[:2] == pytest.approx(prd0[:2], rel=1e-12)
    lam0 = (x - lo) / prd0
    lam = (atom.x.to_numpy()[:n] - dom.boxlo) / prd
    assert np.abs(lam - lam0).max() < 1e-9


def test_remap_keeps_fraction(gpu):
    """tests/test_deform_pressure.py:223-256 on the GPU path (1e-12)."""
    import taichimps_gb300 as G
    BOX, DT = 0.02, 1.0e-6
    domain = G.Domain(boxlo=[0.0] * 3, boxhi=[BOX] * 3, boundary=("p", "p", "p"))
    atom = G.AtomSystem(max_atoms=2)
    atom.add_particles(x=np.array([[0.5 * BOX] * 3, [0.25 * BOX] * 3]), radius=1e-4, density=2650.0)
    fix = G.FixDeformPressure(domain=domain, axes={d: {"style": "erate", "rate": -1.0e3} for d in "xyz"}, nevery=1)
    fix.setup(0)
    for _ in range(50):
        fix.end_of_step(atom, DT)
    domain.pull()
    prd = np.array(domain.prd)
    lo = np.array(domain.boxlo)
    pos = atom.x.to_numpy()[:2]
    assert prd[0] < BOX
    np.testing.assert_allclose((pos[0] - lo) / prd, [0.5] * 3, atol=1e-12)
    np.testing.assert_allclose((pos[1] - lo) / prd, [0.25] * 3, atol=1e-12)


def test_pbc_and_stale_box(gpu):
    """tests/test_domain_neighbor.py:15-31 and test_lammps_parity.py:128-150."""
    import taichimps_gb300 as G
    domain = G.Domain(boxlo=[0.0] * 3, boxhi=[10.0] * 3, boundary=["p", "p", "p"])
    atom = G.AtomSystem(max_atoms=10)
    atom.add_particles(tag=[1], atom_type=[1], x=[[10.5, -0.2, 5.0]], radius=[0.5], density=[1000.0])
    domain.pbc(atom)
    x = atom.x.to_numpy()[0]
    assert np.isclose(x[0], 0.5) and np.isclose(x[1], 9.8)
    domain.set_box([0.0] * 3, [4.0, 10.0, 10.0])
    atom2 = G.AtomSystem(max_atoms=1)
    atom2.add_particles(x=[[9.5, 1.0, 1.0]], radius=0.1, density=1000.0)
    domain.pbc(atom2)
    np.testing.assert_allclose(atom2.x.to_numpy()[0][0], 1.5, atol=1e-12)


def test_friction_damps_spin(gpu):
    """tests/test_lammps_parity.py:159-190 on the GPU path."""
    import taichimps_gb300 as G
    radius, overlap, spin = 0.5, 0.01, 3.0
    d = 2.0 * radius - overlap
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[6.0] * 3)
    atom = G.AtomSystem(max_atoms=8)
    atom.add_particles(x=[[3.0, 3.0, 3.0], [3.0 + d, 3.0, 3.0]], radius=radius, density=2650.0,
                       omega=np.array([[0.0, 0.0, spin], [0.0, 0.0, 0.0]]))
    nl = G.NeighborList(domain=dom, max_atoms=8, max_neighbors_per_atom=32, skin=0.1)
    hist = G.ContactHistory(max_atoms=8, max_neighbors=32)
    pair = G.GranHookeHistory(domain=dom, kn=1.0e5, gamman=10.0, kt=5.0e4, gammat=5.0, xmu=0.5)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=1e-4)
    sim.add_fix(G.FixNVESphere(domain=dom))
    sim.init_simulation()
    sim.step()
    f = atom.f.to_numpy()[:2]
    t = atom.torque.to_numpy()[:2]
    assert f[0][1] < 0.0 and t[0][2] < 0.0
    np.testing.assert_allclose(f[0] + f[1], np.zeros(3), atol=1e-12 * np.abs(f).max())


def test_pressure_translation_invariant(gpu):
    """tests/test_lammps_parity.py:153-177 on the GPU path."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(7)
    box = 6.0
    radius = 0.52 * (box / 4)
    side = 4
    sp = box / side
    pts = np.array([[(a + 0.5) * sp, (b + 0.5) * sp, (c + 0.5) * sp] for a in range(side) for b in range(side)
                    for c in range(side)])
    pts = (pts + rng.uniform(-0.02 * sp, 0.02 * sp, size=pts.shape)) % box
    computes = G.Computes()

    def p_for(offset):
        dom = G.Domain(boxlo=[0.0] * 3, boxhi=[box] * 3)
        atom = G.AtomSystem(max_atoms=64)
        atom.add_particles(x=(pts + offset) % box, radius=radius, density=2650.0)
        nl = G.NeighborList(domain=dom, max_atoms=64, max_neighbors_per_atom=32, skin=0.1)
        hist = G.ContactHistory(max_atoms=64, max_neighbors=32)
        pair = G.GranHookeHistory(domain=dom, kn=1.0e5, gamman=10.0, kt=5.0e4, gammat=5.0, xmu=0.5)
        sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=1e-4)
        sim.add_fix(G.FixNVESphere(domain=dom))
        sim.init_simulation()
        return computes.compute_pressure_tensor(atom, dom, kinetic=False)

    p0 = p_for(np.zeros(3))
    p1 = p_for(np.array([0.37 * box, 0.11 * box, 0.53 * box]))
    assert np.linalg.norm(p0) > 0.0
    np.testing.assert_allclose(p1, p0, rtol=1e-9, atol=1e-6 * np.linalg.norm(p0))


def test_box_nonpositive_raises(gpu):
    """A servo that collapses the box raises the reference's error (deform_pressure.py:1167-1171)."""
    import taichimps_gb300 as G
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[1.0] * 3)
    atom = G.AtomSystem(max_atoms=1)
    atom.add_particles(x=[[0.5, 0.5, 0.5]], radius=0.1, density=1.0)
    nl = G.NeighborList(domain=dom, max_atoms=1, max_neighbors_per_atom=4, skin=0.1)
    hist = G.ContactHistory(max_atoms=1, max_neighbors=4)
    pair = G.GranHooke(domain=dom, kn=1.0, gamman=0.0, kt=0.0, gammat=0.0, xmu=0.0)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=1.0)
    sim.add_fix(G.FixDeformPressure(domain=dom, axes={"x": {"style": "erate", "rate": -0.6}}))
    with pytest.raises(RuntimeError, match="not positive"):
        sim.run(5)


def test_empty_system(gpu):
    import taichimps_gb300 as G
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[5.0] * 3)
    atom = G.AtomSystem(max_atoms=4)
    nl = G.NeighborList(domain=dom, max_atoms=4, skin=0.1)
    hist = G.ContactHistory(max_atoms=4)
    pair = G.GranHookeHistory(domain=dom, kn=1.0, gamman=0.0, kt=1.0, gammat=0.0, xmu=0.5)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=1e-3)
    sim.add_fix(G.FixNVESphere(domain=dom))
    sim.run(3)
    assert atom.nlocal == 0
