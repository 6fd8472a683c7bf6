"""
GPU contact kernel vs the oracle, FP64 form: per-call forces, torques and the
per-atom virial within 1e-12 relative (max-abs normalised, the form of the
reference's LAMMPS comparison, tests/test_lammps_reference.py:134-141), for
every pair style, over several calls so the shear history is exercised.
"""

import numpy as np
import pytest

from _twin import PAIR_STYLES, dense_packing, gpu_pair, oracle_pair, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _setup(O, name, seed=0, n=343, box=7.0, boundary=("p", "p", "p")):
    import taichimps_gb300 as G
    rng = np.random.default_rng(seed)
    x, r = dense_packing(rng, n, box, 0.5, 0.58)
    v = rng.normal(scale=0.3, size=(n, 3))
    w = rng.normal(scale=1.0, size=(n, 3))
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[box] * 3, boundary=boundary)
    atom = G.AtomSystem(max_atoms=n)
    atom.add_particles(x=x, radius=r, density=2.5, v=v, omega=w)
    nl = G.NeighborList(domain=dom, skin=0.1, max_atoms=n, max_neighbors_per_atom=32)
    hist = G.ContactHistory(max_atoms=n, max_neighbors=32)
    nl.build(atom)
    hist.restore_state(atom, nl)
    pair = gpu_pair(name, dom)
    odom = O.OracleDomain.make([0.0] * 3, [box] * 3, boundary)
    oat = O.OracleAtoms(x=x, radius=r, density=2.5, v=v, omega=w)
    onl = O.OracleNeighbor(odom, skin=0.1, max_neighbors=32)
    onl.build(oat)
    oh = O.OracleHistory(32)
    oh.restore_state(oat, onl)
    return atom, nl, hist, pair, oat, onl, oh, oracle_pair(O, name), odom


@pytest.mark.parametrize("name", list(PAIR_STYLES))
@pytest.mark.parametrize("boundary", [("p", "p", "p"), ("f", "p", "f")])
def test_forces_match_oracle(gpu, oracle, name, boundary):
    atom, nl, hist, pair, oat, onl, oh, opair, odom = _setup(oracle, name, boundary=boundary)
    n = atom.nlocal
    dt = 1e-4
    for call in range(4):
        upd = call != 0  # first call as the setup evaluation (shearupdate=False)
        atom.clear_forces()
        pair.compute(atom, nl, hist, dt, shearupdate=upd)
        oat.clear_forces()
        opair.compute(oat, onl, oh, odom, dt, shearupdate=upd)
        assert np.abs(oat.f).max() > 0.0
        for fld, ref in (("f", oat.f), ("torque", oat.torque), ("virial", oat.virial)):
            got = getattr(atom, fld).to_numpy()[:n]
            assert rel_err(got, ref) < TOL, (fld, call, rel_err(got, ref))
    # shear history: every touching contact, both sides, in each row atom's own sense
    if pair.uses_history:
        g = hist.contacts_by_tag(nl)
        ref = oh.touching(oat, onl)
        assert set(ref).issubset(set(g))
        scale = max(np.abs(s).max() for s in ref.values())
        assert scale > 0.0
        for (ti, tj), s in ref.items():
            assert np.abs(g[(ti, tj)] - s).max() <= TOL * scale
            np.testing.assert_array_equal(g[(tj, ti)], -g[(ti, tj)])


def test_hooke_known_answer_gpu(gpu):
    """tests/test_hooke.py:16-55 through the GPU path: 4288.790204786391, rtol 1e-12."""
    import taichimps_gb300 as G
    dom = G.Domain(boxlo=[-10.0] * 3, boxhi=[10.0] * 3, boundary=["f", "f", "f"])
    atom = G.AtomSystem(max_atoms=10)
    atom.add_particles(tag=[1, 2], atom_type=[1, 1], x=[[0.0, 0.0, 0.0], [1.9, 0.0, 0.0]],
                       v=[[0.1, 0.0, 0.0], [-0.1, 0.0, 0.0]], radius=[1.0, 1.0], density=[1000.0, 1000.0])
    nl = G.NeighborList(domain=dom, skin=0.2, max_atoms=10, max_neighbors=10)
    nl.build(atom)
    history = G.ContactHistory(max_atoms=10, max_neighbors=10)
    pair = G.GranHooke(domain=dom, kn=1000.0, gamman=10.0, kt=0.0, gammat=0.0, xmu=0.0, dampflag=0)
    pair.compute(atom, nl, history, dt=0.001)
    expected = 4288.790204786391
    f = atom.f.to_numpy()
    np.testing.assert_allclose(f[0], [-expected, 0.0, 0.0], rtol=1e-12)
    np.testing.assert_allclose(f[1], [expected, 0.0, 0.0], rtol=1e-12)


def test_history_pair_view(gpu):
    """The reference-style per-pair view (partner tags, i->j shear) of a touching pair."""
    import taichimps_gb300 as G
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[10.0] * 3)
    atom = G.AtomSystem(max_atoms=10)
    atom.add_particles(tag=[1, 2], x=[[1.0, 0.0, 0.0], [2.9, 0.0, 0.0]], v=[[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]],
                       radius=[1.0, 1.0], density=[1000.0, 1000.0])
    nl = G.NeighborList(domain=dom, max_atoms=10, max_neighbors=5, skin=0.2)
    hist = G.ContactHistory(max_atoms=10, max_neighbors=5)
    nl.build(atom)
    pair = G.GranHookeHistory(domain=dom, kn=1000.0, gamman=0.0, kt=500.0, gammat=0.0, xmu=0.5)
    pair.compute(atom=atom, nlist=nl, history=hist, dt=0.001)
    f = atom.f.to_numpy()
    assert f[0, 1] < 0.0 < f[1, 1]
    assert np.isclose(f[0, 1], -f[1, 1])
    assert list(hist.partner) == [2]
    sh = hist.shear_pairs[0]
    assert sh[1] == pytest.approx(0.002)  # vtr_y * dt with vtr = v_i - v_j = +2
