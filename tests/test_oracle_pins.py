"""
Pins the CPU oracle to the reference's own known answers and invariants.

Each test restates a reference test (taichimps/tests/...) against the oracle,
with the reference's inputs and tolerances, so that the oracle the GPU path is
checked against is itself checked before it is trusted.
"""

import json
import math
from pathlib import Path

import numpy as np
import pytest

# literal inputs and expected values of the reference's tests (tests/golden/make_known_answers.py)
GOLDEN = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())["cases"]


def _two_sphere_hooke(O):
    c = GOLDEN["hooke_normal_contact"]
    d, p = c["domain"], c["particles"]
    dom = O.OracleDomain.make(d["boxlo"], d["boxhi"], tuple(d["boundary"]))
    atoms = O.OracleAtoms(x=p["x"], v=p["v"], radius=p["radius"], density=p["density"], tag=p["tag"])
    nl = O.OracleNeighbor(dom, skin=c["skin"], max_neighbors=10)
    nl.build(atoms)
    hist = O.OracleHistory(10)
    hist.restore_state(atoms, nl)
    return dom, atoms, nl, hist


def test_hooke_known_answer(oracle):
    """tests/test_hooke.py:16-55: F = 4288.790204786391 (LAMMPS-verified), rtol 1e-12."""
    O = oracle
    c = GOLDEN["hooke_normal_contact"]
    dom, atoms, nl, hist = _two_sphere_hooke(O)
    pair = O.OraclePair("hooke", **c["pair"])
    pair.compute(atoms, nl, hist, dom, dt=c["dt"])
    fx0, fx1 = c["expected_fx"]
    np.testing.assert_allclose(atoms.f[0], [fx0, 0.0, 0.0], rtol=c["rtol"])
    np.testing.assert_allclose(atoms.f[1], [fx1, 0.0, 0.0], rtol=c["rtol"])


def _random_packing(rng, n=60, box=6.0):
    """tests/test_lammps_parity.py:112-125: jittered lattice dense enough to overlap."""
    side = int(np.ceil(n ** (1.0 / 3.0)))
    spacing = box / side
    pts = []
    for ix in range(side):
        for iy in range(side):
            for iz in range(side):
                if len(pts) >= n:
                    break
                pts.append([(ix + 0.5) * spacing, (iy + 0.5) * spacing, (iz + 0.5) * spacing])
    pts = np.asarray(pts[:n], dtype=np.float64)
    pts += rng.uniform(-0.02 * spacing, 0.02 * spacing, size=pts.shape)
    return pts % box


def _parity_sim(O, positions, radius, box=6.0, skin=0.1, xmu=0.5, v=None, w=None, dt=1e-4):
    """tests/test_lammps_parity.py:89-109"""
    dom = O.OracleDomain.make([0.0] * 3, [box] * 3)
    atoms = O.OracleAtoms(x=positions, radius=radius, density=2650.0, v=v, omega=w)
    nl = O.OracleNeighbor(dom, skin=skin, max_neighbors=32)
    hist = O.OracleHistory(32)
    pair = O.OraclePair("hooke/history", kn=1.0e5, gamman=10.0, kt=5.0e4, gammat=5.0, xmu=xmu)
    return O.OracleSim(dom, atoms, nl, hist, pair, dt)


def test_pressure_translation_invariant(oracle):
    """tests/test_lammps_parity.py:153-177: pair virial independent of the origin, rtol 1e-9."""
    O = oracle
    rng = np.random.default_rng(7)
    box = 6.0
    radius = 0.52 * (box / 4)
    pts = _random_packing(rng, n=64, box=box)

    def p_for(offset):
        sim = _parity_sim(O, (pts + offset) % box, radius, box=box)
        sim.setup()
        return O.pressure_tensor(sim.atoms, sim.domain, kinetic=False)

    p0 = p_for(np.zeros(3))
    p1 = p_for(np.array([0.37 * box, 0.11 * box, 0.53 * box]))
    assert np.linalg.norm(p0) > 0.0
    np.testing.assert_allclose(p1, p0, rtol=1e-9, atol=1e-6 * np.linalg.norm(p0))


def test_shear_history_survives_rebuild(oracle):
    """tests/test_lammps_parity.py:124-157: rebuild every step == never rebuild, rtol 1e-8."""
    O = oracle
    rng = np.random.default_rng(11)
    box = 6.0
    radius = 0.52 * (box / 4)
    pts = _random_packing(rng, n=64, box=box)
    vel = rng.normal(scale=0.05, size=pts.shape)
    omg = rng.normal(scale=0.5, size=pts.shape)

    def run(every_step):
        sim = _parity_sim(O, pts, radius, box=box, v=vel, w=omg)
        if every_step:
            sim.neighbor.check, sim.neighbor.every = False, 1
        else:
            sim.neighbor.check, sim.neighbor.every = True, 10 ** 6
        sim.run(40)
        return sim.atoms.f.copy()

    f_re, f_keep = run(True), run(False)
    scale = np.abs(f_keep).max()
    assert scale > 0.0
    np.testing.assert_allclose(f_re, f_keep, rtol=1e-8, atol=1e-8 * scale)


def test_friction_damps_spin(oracle):
    """tests/test_lammps_parity.py:159-190: friction opposes spin; Newton's third law."""
    O = oracle
    radius, overlap, spin = 0.5, 0.01, 3.0
    d = 2.0 * radius - overlap
    sim = _parity_sim(O, [[3.0, 3.0, 3.0], [3.0 + d, 3.0, 3.0]], radius,
                      w=np.array([[0.0, 0.0, spin], [0.0, 0.0, 0.0]]))
    sim.setup()
    sim.step()
    f, t = sim.atoms.f, sim.atoms.torque
    assert f[0][1] < 0.0
    assert t[0][2] < 0.0
    np.testing.assert_allclose(f[0] + f[1], np.zeros(3), atol=1e-12 * np.abs(f).max())


def test_pbc_wrap(oracle):
    """tests/test_domain_neighbor.py:15-31: 10.5 -> 0.5, -0.2 -> 9.8."""
    import ctypes
    O = oracle
    c = GOLDEN["pbc_wrap"]
    d = c["domain"]
    dom = O.OracleDomain.make(d["boxlo"], d["boxhi"], tuple(d["boundary"]))
    x = np.array(c["particles"]["x"], dtype=np.float64)
    v = np.zeros((1, 3))
    O.lib().or_pbc(ctypes.byref(dom.cbox()), 1, O._p(x), O._p(v))
    assert 0.0 <= x[0, 0] < 10.0 and 0.0 <= x[0, 1] < 10.0
    for k, val in c["expected"].items():
        assert np.isclose(x[0, int(k)], val)


def test_neighbor_list_and_skin_trigger(oracle):
    """tests/test_domain_neighbor.py:34-92: neighbor set; skin 0.2 -> 0.08 no, 0.12 yes."""
    O = oracle
    dom = O.OracleDomain.make([-10.0] * 3, [10.0] * 3, ("f", "f", "f"))
    atoms = O.OracleAtoms(x=[[0, 0, 0], [1.5, 0, 0], [5.0, 0, 0]], radius=[1.0] * 3, density=[1000.0] * 3)
    nl = O.OracleNeighbor(dom, skin=0.2, max_neighbors=10)
    assert nl.decide(atoms, 0)
    nl.build(atoms)
    assert nl.num_neighbors[0] == 1 and nl.neighbors[0, 0] == 1
    assert not nl.decide(atoms, 1)
    atoms.x[0] = [0.08, 0.0, 0.0]
    assert not nl.decide(atoms, 2)
    atoms.x[0] = [0.12, 0.0, 0.0]
    assert nl.decide(atoms, 3)


def test_remap_x_affine(oracle):
    """tests/test_deform_remap_x.py:24-111: erate -0.05 on z, remap x, 30 steps."""
    O = oracle
    RADIUS, DENSITY, DT, ERATE = 5.0e-4, 2650.0, 1.0e-7, -0.05
    n_side = 6
    lo, hi = 0.0, n_side * 2.5 * RADIUS
    g = (np.arange(n_side) + 0.5) * (hi - lo) / n_side
    x = np.array([[a, b, c] for a in g for b in g for c in g])
    dom = O.OracleDomain.make([lo] * 3, [hi] * 3)
    atoms = O.OracleAtoms(x=x, radius=RADIUS, density=DENSITY)
    nl = O.OracleNeighbor(dom, skin=0.4 * RADIUS, max_neighbors=32)
    hist = O.OracleHistory(32)
    pair = O.OraclePair("hertz/history", kn=1e8, gamman=0.0, kt=1e8, gammat=0.0, xmu=0.3, dampflag=0)
    fix = O.OracleDeform(dom, axes={"z": {"style": "erate", "rate": ERATE}}, remap="x")
    sim = O.OracleSim(dom, atoms, nl, hist, pair, DT, fixes=[fix])
    sim.run(30)
    prd0, prd = np.full(3, hi - lo), dom.prd
    assert prd[2] == pytest.approx(prd0[2] * (1.0 + ERATE * 30 * DT), rel=1e-9)
    assert prd[:2] == pytest.approx(prd0[:2], rel=1e-12)
    lam0 = (x - lo) / prd0
    lam = (atoms.x - dom.boxlo) / prd
    assert np.abs(lam - lam0).max() < 1e-9


def test_remap_keeps_fraction(oracle):
    """tests/test_deform_pressure.py:223-256: 50 erate updates keep fractional coordinates (1e-12)."""
    O = oracle
    BOX, DT = 0.02, 1.0e-6
    dom = O.OracleDomain.make([0.0] * 3, [BOX] * 3)
    atoms = O.OracleAtoms(x=[[0.5 * BOX] * 3, [0.25 * BOX] * 3], radius=1e-4, density=2650.0)
    fix = O.OracleDeform(dom, axes={d: {"style": "erate", "rate": -1.0e3} for d in "xyz"})
    fix.setup(0, DT, 2)
    for _ in range(50):
        fix.end_of_step(atoms, DT)
    prd, lo = dom.prd, dom.boxlo
    assert prd[0] < BOX
    np.testing.assert_allclose((atoms.x[0] - lo) / prd, [0.5] * 3, atol=1e-12)
    np.testing.assert_allclose((atoms.x[1] - lo) / prd, [0.25] * 3, atol=1e-12)


def test_sign_checks(oracle):
    """tests/test_additional_models.py:15-97: tangential and Hertz force signs."""
    O = oracle
    dom = O.OracleDomain.make([0.0] * 3, [10.0] * 3)
    atoms = O.OracleAtoms(x=[[1.0, 0, 0], [2.9, 0, 0]], v=[[0, 1.0, 0], [0, -1.0, 0]], radius=[1.0, 1.0],
                          density=[1000.0, 1000.0])
    nl = O.OracleNeighbor(dom, skin=0.2, max_neighbors=5)
    nl.build(atoms)
    hist = O.OracleHistory(5)
    hist.restore_state(atoms, nl)
    O.OraclePair("hooke/history", kn=1000.0, gamman=0.0, kt=500.0, gammat=0.0, xmu=0.5).compute(
        atoms, nl, hist, dom, 0.001)
    assert atoms.f[0, 1] < 0.0 < atoms.f[1, 1]
    assert np.isclose(atoms.f[0, 1], -atoms.f[1, 1])
    atoms2 = O.OracleAtoms(x=[[1.0, 0, 0], [2.9, 0, 0]], radius=[1.0, 1.0], density=[1000.0, 1000.0])
    nl2 = O.OracleNeighbor(dom, skin=0.2, max_neighbors=5)
    nl2.build(atoms2)
    h2 = O.OracleHistory(5)
    h2.restore_state(atoms2, nl2)
    O.OraclePair("hertz", kn=1000.0, gamman=0.0, kt=0.0, gammat=0.0, xmu=0.0).compute(atoms2, nl2, h2, dom, 0.001)
    assert atoms2.f[0, 0] < 0.0 < atoms2.f[1, 0]


def test_granular_derived_coefficients(oracle):
    """tests/test_pair_granular_parsing.py:56-85: derived kn, kt and damp, rtol 1e-12."""
    O = oracle
    EMOD, POISS, COR, FRIC = 71.6e9, 0.23, 0.95, 0.3
    p = O.OraclePair("granular", normal="hertz/material", normal_coeffs=[EMOD, COR, POISS],
                     tangential="mindlin", tangential_coeffs=[None, 1.0, FRIC], damping="coeff_restitution")
    e_eff = 1.0 / ((1 - POISS ** 2) / EMOD * 2)
    g_eff = 1.0 / (2 * (2 - POISS) * (1 + POISS) / EMOD * 2)
    np.testing.assert_allclose(p.P.kn, 4.0 / 3.0 * e_eff, rtol=1e-12)
    np.testing.assert_allclose(p.P.kt, 8.0 * g_eff, rtol=1e-12)
    logcor = math.log(COR)
    damp = -1.22474487139158894067 * 1.82574185835055380345 * logcor / math.sqrt(math.pi ** 2 + logcor ** 2)
    np.testing.assert_allclose(p.P.damp, damp, rtol=1e-12)
    assert p.P.mu == pytest.approx(FRIC)


def test_pair_antisymmetry_all_styles(oracle):
    """Every pair law is exactly odd under i <-> j: evaluating a contact in either
    orientation gives bitwise the same force and torque on each atom.  The GPU
    full list relies on this (each contact is evaluated by both of its atoms)."""
    O = oracle
    rng = np.random.default_rng(3)
    styles = [("hooke", {}), ("hooke/history", {}), ("hertz", {}), ("hertz/history", {}),
              ("granular", dict(normal="hertz/material", normal_coeffs=[5e6, 0.5, 0.3], tangential="mindlin",
                                tangential_coeffs=[None, 1.0, 0.5], damping="coeff_restitution")),
              ("granular", dict(normal="hooke", normal_coeffs=[2e5, 30.0], tangential="linear_history",
                                tangential_coeffs=[5e4, 0.5, 0.4], damping="mass_velocity")),
              ("granular", dict(normal="hertz", normal_coeffs=[2e5, 10.0], tangential="linear_nohistory",
                                tangential_coeffs=[0.5, 0.4], damping="viscoelastic")),
              ("granular", dict(normal="hertz/material", normal_coeffs=[5e6, 0.5, 0.3], tangential="mindlin",
                                tangential_coeffs=[None, 1.0, 0.5], damping="coeff_restitution",
                                rolling="epsd", rolling_coeffs=[1e3, 50.0, 0.1]))]
    x = np.array([[1.0, 1.0, 1.0], [1.95, 1.1, 0.97]])
    rad = np.array([0.5, 0.52])
    v = rng.normal(size=(2, 3))
    w = rng.normal(size=(2, 3))
    for style, kw in styles:
        base = dict(kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5) if style != "granular" else kw
        res = []
        for order in ([0, 1], [1, 0]):
            dom = O.OracleDomain.make([0.0] * 3, [5.0] * 3)
            atoms = O.OracleAtoms(x=x[order], v=v[order], omega=w[order], radius=rad[order], density=2.5,
                                  tag=np.array([1, 2])[order])
            nl = O.OracleNeighbor(dom, skin=0.1, max_neighbors=8)
            nl.build(atoms)
            hist = O.OracleHistory(8)
            hist.restore_state(atoms, nl)
            pair = O.OraclePair(style, **base)
            for _ in range(3):
                atoms.clear_forces()
                pair.compute(atoms, nl, hist, dom, 1e-4)
            back = np.argsort(order)
            res.append((atoms.f[back].copy(), atoms.torque[back].copy(), atoms.virial[back].copy()))
        assert np.abs(res[0][0]).max() > 0.0
        for a, b in zip(res[0], res[1]):
            np.testing.assert_array_equal(a, b)


def test_contact_count_brute_force(oracle):
    """computes/contact_atom.py:21-52 restated in the oracle: the per-atom contact counts equal an
    all-pairs count with the minimum image (each contact counted for both partners)."""
    O = oracle
    rng = np.random.default_rng(12)
    box = 6.0
    x = _random_packing(rng, n=64, box=box)
    r = rng.uniform(0.7, 0.85, size=len(x))
    dom = O.OracleDomain.make([0.0] * 3, [box] * 3)
    atoms = O.OracleAtoms(x=x, radius=r, density=2.5)
    nl = O.OracleNeighbor(dom, skin=0.1, max_neighbors=32)
    nl.build(atoms)
    got = nl.contact_count(atoms)
    d = x[:, None, :] - x[None, :, :]
    d -= box * np.where(np.abs(d / box) % 1 == 0.5, np.sign(d / box) * np.ceil(np.abs(d / box)), np.round(d / box))
    rsq = (d ** 2).sum(-1)
    rs = r[:, None] + r[None, :]
    want = ((rsq < rs * rs) & (rsq > 1e-18)).sum(1)
    assert got.sum() > 0
    np.testing.assert_array_equal(got, want)


def test_rolling_resistance_torque(oracle):
    """GRANULAR/rolling.py:30-50 (EPSD) in the oracle's pair granular: for two touching spheres at rest
    with a relative spin, the first update gives torque_i = -k h - gamma w_rel with h = w_rel dt on atom i
    and the opposite on atom j (uncapped), added to the tangential torque; the rolling history is
    h; with mu_roll = 0 the cap rescales the history as rolling.py writes it."""
    O = oracle
    x = np.array([[1.0, 1.0, 1.0], [1.9, 1.0, 1.0]])
    rad = np.array([0.5, 0.5])
    w = np.array([[0.0, 0.0, 2.0], [0.0, 0.0, -1.0]])
    dt = 1e-3
    kroll, groll = 1e3, 50.0
    out = {}
    for mu_roll in (1e6, 0.0):
        for rolling in ("none", "epsd"):
            dom = O.OracleDomain.make([0.0] * 3, [5.0] * 3)
            atoms = O.OracleAtoms(x=x, omega=w, radius=rad, density=2.5, tag=[1, 2])
            nl = O.OracleNeighbor(dom, skin=0.1, max_neighbors=8)
            nl.build(atoms)
            hist = O.OracleHistory(8)
            hist.restore_state(atoms, nl)
            kw = dict(normal="hertz/material", normal_coeffs=[5e6, 0.5, 0.3], tangential="mindlin",
                      tangential_coeffs=[None, 1.0, 0.5], damping="coeff_restitution")
            if rolling != "none":
                kw.update(rolling="epsd", rolling_coeffs=[kroll, groll, mu_roll])
            pair = O.OraclePair("granular", **kw)
            atoms.clear_forces()
            pair.compute(atoms, nl, hist, dom, dt)
            out[(mu_roll, rolling)] = (atoms.torque.copy(), hist.rolling[0].copy())
    wrel = w[0] - w[1]
    h = wrel * dt
    troll = -kroll * h - groll * wrel
    t_none, _ = out[(1e6, "none")]
    t_roll, h_got = out[(1e6, "epsd")]
    np.testing.assert_allclose(t_roll[0] - t_none[0], troll, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(t_roll[1] - t_none[1], -troll, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(h_got, h, rtol=1e-15)
    # mu_roll = 0: tr_max = 0 < tr_mag, so torque = 0 and the history is rescaled to zero
    t_cap, h_cap = out[(0.0, "epsd")]
    np.testing.assert_allclose(t_cap, out[(0.0, "none")][0], rtol=1e-15, atol=0)
    np.testing.assert_array_equal(h_cap, np.zeros(3))


WALL_CASES = [k for k in GOLDEN if k.startswith("wall_region_")]


@pytest.mark.parametrize("case", WALL_CASES)
def test_wall_region_known_answers(oracle, case):
    """The reference's cylinder-wall known answers (tests/test_wall_region.py): one post_force call on
    one particle; the reference asserts at rtol 1e-4."""
    c = GOLDEN[case]
    at = oracle.OracleAtoms(x=[c["x"]], radius=c["radius"], density=1.0, v=[c["v"]])
    at.rmass[:] = c["rmass"]
    fix = oracle.OracleWallGranRegion(**c["fix"])
    fix.post_force(at, c["dt"])
    got = {"f_res": at.f[0], "torque_res": at.torque[0]}
    for e in c["expected"]:
        assert got[e["of"]][e["k"]] == pytest.approx(e["value"], rel=1e-4, abs=1e-5), e


def test_wall_plane_known_sign(oracle):
    """tests/test_additional_models.py: a particle overlapping a plane wall at x = 0 is pushed away."""
    c = GOLDEN["wall_plane_sign"]
    p = c["particles"]
    at = oracle.OracleAtoms(x=p["x"], radius=p["radius"], density=p["density"], v=p["v"])
    fix = oracle.OracleWallGran(**c["fix"])
    fix.post_force(at, c["dt"])
    assert np.sign(at.f[0, 0]) == c["expected_sign_fx"]
    # hooke, no damping: kn * (r - x)
    assert at.f[0, 0] == pytest.approx(c["fix"]["kn"] * (p["radius"][0] - p["x"][0][0]), rel=1e-12)


def test_wall_history_sticks_then_slides(oracle):
    """Plane wall, hooke/history: the shear spring grows while the tangential force is under the Coulomb
    bound, then the force saturates at xmu |fn| and the spring is rescaled to match (wall_gran.py:196-212)."""
    at = oracle.OracleAtoms(x=[[0.5, 0.5, 0.09]], radius=0.1, density=1.0, v=[[1.0, 0.0, 0.0]])
    fix = oracle.OracleWallGran(wall_axis=2, wall_side=-1, wall_coord=0.0, kn=1e4, gamman=0.0, kt=2e3,
                                gammat=0.0, xmu=0.5)
    fts = []
    for _ in range(40):
        at.f[:] = 0.0
        fix.post_force(at, 1e-2)
        fts.append(at.f[0, 0])
    fn = 1e4 * 0.01
    assert fts[0] == pytest.approx(-2e3 * 1.0 * 1e-2, rel=1e-12)   # kt |v| dt while sticking
    assert fts[1] == pytest.approx(2.0 * fts[0], rel=1e-12)
    assert fts[2] == pytest.approx(-0.5 * fn, rel=1e-12)          # capped at xmu |fn|
    assert fts[-1] == pytest.approx(-0.5 * fn, rel=1e-12)
    assert np.linalg.norm(fix.shear[0]) == pytest.approx(0.5 * fn / 2e3, rel=1e-12)
