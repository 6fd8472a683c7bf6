"""
Granular walls on the GPU (taichimps_gb300/EXTRA_FIX/wall_gran.py, wall_gran_region.py,
csrc/tmps_wall.cu): the reference's known answers (tests/golden), then whole runs
against the oracle -- plane walls with and without history, a shearing and a
wiggling wall, the inside and outside of a cylinder with hooke and hertz,
axis bounds -- with pair contacts, nve/sphere and neighbor rebuilds (the wall
history follows the atoms through the build's re-sort).
"""

import json
from pathlib import Path

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin, oracle_state, rel_err

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())["cases"]


def _one_atom(G, x, v, radius, rmass):
    dom = G.Domain(boxlo=[-2.0] * 3, boxhi=[2.0] * 3, boundary=("f", "f", "f"))
    atom = G.AtomSystem(max_atoms=4)
    dens = rmass / ((4.0 / 3.0) * np.pi * radius ** 3)
    atom.add_particles(x=[x], v=[v], radius=[radius], density=[dens])
    atom.clear_forces()
    return dom, atom


@pytest.mark.parametrize("case", [k for k in GOLDEN if k.startswith("wall_region_")])
def test_wall_region_known_answers(gpu, case):
    import taichimps_gb300 as G
    c = GOLDEN[case]
    dom, atom = _one_atom(G, c["x"], c["v"], c["radius"], c["rmass"])
    fix = G.FixWallGranRegion(domain=dom, max_atoms=4, **c["fix"])
    fix.post_force(atom, c["dt"])
    got = {"f_res": atom.f.to_numpy()[0], "torque_res": atom.torque.to_numpy()[0]}
    for e in c["expected"]:
        assert got[e["of"]][e["k"]] == pytest.approx(e["value"], rel=1e-4, abs=1e-5), e


def test_wall_plane_known_sign(gpu):
    import taichimps_gb300 as G
    c = GOLDEN["wall_plane_sign"]
    p = c["particles"]
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[10.0] * 3)
    atom = G.AtomSystem(max_atoms=4)
    atom.add_particles(x=p["x"], v=p["v"], radius=p["radius"], density=p["density"])
    atom.clear_forces()
    fix = G.FixWallGran(domain=dom, max_atoms=4, **c["fix"])
    fix.post_force(atom, c["dt"])
    f = atom.f.to_numpy()
    assert np.sign(f[0, 0]) == c["expected_sign_fx"]
    assert f[0, 0] == pytest.approx(c["fix"]["kn"] * (p["radius"][0] - p["x"][0][0]), rel=1e-12)


def _run_pair(oracle, walls, boundary, box, v_scale=1.5, steps=300, seed=3, w_scale=3.0, keep=None):
    import taichimps_gb300 as G
    rng = np.random.default_rng(seed)
    x, r = dense_packing(rng, 216, box, 0.42, 0.5, jitter=0.05)
    if keep is not None:
        m = keep(x, r)
        x, r = x[m], r[m]
    v = rng.normal(scale=v_scale, size=x.shape)
    w = rng.normal(scale=w_scale, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, boundary=boundary, v=v, w=w,
                          pair="hooke/history", dt=1e-4, skin=0.05)
    for kind, kw in walls:
        if kind == "plane":
            sim.add_fix(G.FixWallGran(domain=sim.domain, max_atoms=len(x), **kw))
            osim.fixes.append(oracle.OracleWallGran(**kw))
        else:
            sim.add_fix(G.FixWallGranRegion(domain=sim.domain, max_atoms=len(x), **kw))
            osim.fixes.append(oracle.OracleWallGranRegion(**kw))
    # 20 steps with the contacts still on the walls: the wall history against the oracle's
    sim.run(20)
    osim.run(20)
    n = len(x)
    for fg, fo in zip(sim.fixes[-len(walls):], osim.fixes[-len(walls):]):
        if fg.use_history:
            sh = fg.shear[:, :n].T.cpu().numpy()   # slots by insertion order, like the oracle's atoms
            assert np.abs(fo.shear).max() > 0
            assert rel_err(sh, fo.shear) < 1e-10, rel_err(sh, fo.shear)
            np.testing.assert_array_equal(fg.touch[:n].cpu().numpy(), fo.touch)
    # a second run without the setup force evaluation (run ... pre no); every run still
    # calls the fixes' setup (simulation.py:161-168), which restarts a wiggling wall's clock
    sim.run_pre = False
    sim.run(steps - 20)
    for fx in osim.fixes:
        if hasattr(fx, "setup"):
            fx.setup(steps - 20, osim.dt, osim.atoms.n)
    for _ in range(steps - 20):
        osim.step()
    return sim, osim


PLANE = dict(kn=2e5, gamman=50.0, kt=2e5 * 2 / 7, gammat=25.0, xmu=0.5)


@pytest.mark.parametrize("variant", ["history", "nohistory", "shear", "wiggle"])
def test_plane_walls_match_oracle(gpu, oracle, variant):
    box = 6.0
    lo = dict(wall_axis=2, wall_side=-1, wall_coord=0.0, **PLANE)
    hi = dict(wall_axis=2, wall_side=1, wall_coord=box, **PLANE)
    if variant == "nohistory":
        lo["history"] = hi["history"] = False
    if variant == "shear":
        lo.update(shear_axis=0, shear_vel=0.5)
    if variant == "wiggle":
        hi.update(wiggle_amplitude=0.01, wiggle_period=0.02)
    sim, osim = _run_pair(oracle, [("plane", lo), ("plane", hi)], ("p", "p", "f"), box)
    assert sim.neighbor.build_count > 1
    g, o = gpu_state(sim), oracle_state(osim)
    for k in ("x", "v", "omega", "f", "torque"):
        assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))


@pytest.mark.parametrize("fstyle,side", [("hooke/history", "in"), ("hertz/history", "in"), ("hooke", "in"),
                                         ("hertz/history", "out")])
def test_cylinder_wall_matches_oracle(gpu, oracle, fstyle, side):
    box = 6.0
    R = 2.6 if side == "in" else 1.2
    kw = dict(axis="z", c1=3.0, c2=3.0, radius=R, side=side, fstyle=fstyle,
              kn=2e5, gamman=50.0, xmu=0.5, axis_lo=0.5, axis_hi=5.5)

    def keep(x, r):
        rp = np.hypot(x[:, 0] - 3.0, x[:, 1] - 3.0)
        # on the contact side of the surface, some already touching it
        return (rp + r < R + 0.05) if side == "in" else (rp - r > R - 0.05)

    sim, osim = _run_pair(oracle, [("cyl", kw)], ("f", "f", "p"), box, keep=keep)
    g, o = gpu_state(sim), oracle_state(osim)
    for k in ("x", "v", "omega", "f", "torque"):
        assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
