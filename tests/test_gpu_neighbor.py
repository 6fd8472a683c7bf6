"""
GPU neighbor build vs the oracle: cell assignments and pair sets must be
bit-identical on the same positions (tolerance: none).
"""

import numpy as np
import pytest

from _twin import dense_packing

pytestmark = pytest.mark.gpu


def _build_both(O, x, radius, lo, hi, boundary=("p", "p", "p"), skin=0.1, max_nb=32):
    import taichimps_gb300 as G
    n = len(x)
    dom = G.Domain(boxlo=lo, boxhi=hi, boundary=boundary)
    atom = G.AtomSystem(max_atoms=n)
    atom.add_particles(x=x, radius=radius, density=2.5)
    nl = G.NeighborList(domain=dom, skin=skin, max_atoms=n, max_neighbors_per_atom=max_nb)
    nl.build(atom)
    odom = O.OracleDomain.make(lo, hi, boundary)
    oat = O.OracleAtoms(x=x, radius=radius, density=2.5)
    onl = O.OracleNeighbor(odom, skin=skin, max_neighbors=max_nb)
    onl.build(oat)
    return atom, nl, oat, onl


def _check_identical(atom, nl, oat, onl):
    assert list(nl.grid_dim) == list(onl.grid_dim)
    # cell of every atom, insertion order
    cell_gpu = np.empty(atom.nlocal, dtype=np.int64)
    cell_gpu[atom.uid_host()] = nl.cell_of.cpu().numpy()
    np.testing.assert_array_equal(cell_gpu, onl.cell_of)
    assert nl.pair_set_tags() == onl.pair_set(oat.tag)


def test_config1_packing_bit_exact(gpu, oracle):
    from taichimps_gb300.packing import config1
    p = config1(seed=1)
    L = p["L"]
    atom, nl, oat, onl = _build_both(oracle, p["x"], p["radius"], [0.0] * 3, [L] * 3)
    _check_identical(atom, nl, oat, onl)
    assert len(onl.pair_set(oat.tag)) > 1000


@pytest.mark.parametrize("boundary", [("p", "p", "p"), ("f", "f", "f"), ("p", "f", "p")])
def test_dense_random_bit_exact(gpu, oracle, boundary):
    rng = np.random.default_rng(5)
    x, r = dense_packing(rng, 729, 9.0, 0.45, 0.6)
    atom, nl, oat, onl = _build_both(oracle, x, r, [0.0] * 3, [9.0] * 3, boundary=boundary)
    _check_identical(atom, nl, oat, onl)


@pytest.mark.parametrize("box", [2.5, 3.3, 4.0])
def test_small_periodic_boxes(gpu, oracle, box):
    """One- and two-bin periodic grids (the collapse and skip rules, neighbor.py:165-175, 334-341)."""
    rng = np.random.default_rng(int(box * 10))
    x = rng.uniform(0, box, size=(20, 3))
    r = rng.uniform(0.3, 0.5, size=20)
    atom, nl, oat, onl = _build_both(oracle, x, r, [0.0] * 3, [box] * 3)
    _check_identical(atom, nl, oat, onl)


def test_atoms_outside_box_clamped(gpu, oracle):
    """Atoms beyond a fixed boundary are clamped into the edge bins (neighbor.py:202-205)."""
    rng = np.random.default_rng(9)
    x = rng.uniform(-1.0, 7.0, size=(200, 3))
    r = rng.uniform(0.3, 0.5, size=200)
    atom, nl, oat, onl = _build_both(oracle, x, r, [0.0] * 3, [6.0] * 3, boundary=("f", "f", "f"))
    _check_identical(atom, nl, oat, onl)


def test_reference_three_atom_list(gpu):
    """tests/test_domain_neighbor.py:34-55 on the GPU path."""
    import taichimps_gb300 as G
    dom = G.Domain(boxlo=[-10.0] * 3, boxhi=[10.0] * 3, boundary=["f", "f", "f"])
    atom = G.AtomSystem(max_atoms=10)
    atom.add_particles(tag=[1, 2, 3], atom_type=[1, 1, 1], x=[[0, 0, 0], [1.5, 0, 0], [5.0, 0, 0]],
                       radius=[1.0] * 3, density=[1000.0] * 3)
    nl = G.NeighborList(domain=dom, skin=0.2, max_atoms=10, max_neighbors=10)
    nl.build(atom)
    assert nl.num_neighbors.to_numpy()[0] == 1
    assert nl.neighbors.to_numpy()[0, 0] == 1


def test_skin_trigger(gpu):
    """tests/test_domain_neighbor.py:58-92: 0.08 < skin/2 keeps, 0.12 > skin/2 rebuilds."""
    import taichimps_gb300 as G
    dom = G.Domain(boxlo=[-10.0] * 3, boxhi=[10.0] * 3, boundary=["f", "f", "f"])
    atom = G.AtomSystem(max_atoms=10)
    atom.add_particles(tag=[1, 2, 3], x=[[0, 0, 0], [1.5, 0, 0], [5.0, 0, 0]], radius=[1.0] * 3,
                       density=[1000.0] * 3)
    nl = G.NeighborList(domain=dom, skin=0.2, max_atoms=10, max_neighbors=10)
    assert nl.check_and_build(atom, timestep=0) is True and nl.build_count == 1
    assert nl.check_and_build(atom, timestep=1) is False and nl.build_count == 1
    atom.x[0] = [0.08, 0.0, 0.0]
    assert nl.check_and_build(atom, timestep=2) is False and nl.build_count == 1
    atom.x[0] = [0.12, 0.0, 0.0]
    assert nl.check_and_build(atom, timestep=3) is True and nl.build_count == 2


def test_overflow_raises(gpu):
    """A row that does not fit raises the reference's error (neighbor.py:426-431)."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(2)
    x, r = dense_packing(rng, 216, 4.0, 0.5, 0.6)
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[4.0] * 3)
    atom = G.AtomSystem(max_atoms=216)
    atom.add_particles(x=x, radius=r, density=2.5)
    nl = G.NeighborList(domain=dom, skin=0.1, max_atoms=216, max_neighbors_per_atom=2)
    with pytest.raises(RuntimeError, match="Neighbor list overflow"):
        nl.build(atom)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overflow_raises_through_a_run(gpu, precision):
    """Inside a run the build does not wait for the device: the overflow is read at the run's next
    synchronisation and raised there, before any step's result is handed back; a deferred status is
    read once (a later build or check does not raise it again)."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(2)
    x, r = dense_packing(rng, 216, 4.0, 0.5, 0.6)
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[4.0] * 3)
    atom = G.AtomSystem(max_atoms=216)
    atom.add_particles(x=x, radius=r, density=2.5)
    nl = G.NeighborList(domain=dom, skin=0.1, max_atoms=216, max_neighbors_per_atom=2)
    hist = G.ContactHistory(max_atoms=216, max_neighbors=2)
    pair = G.GranHertzHistory(domain=dom, kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=pair, dt=5e-5, precision=precision)
    sim.add_fix(G.FixNVESphere(domain=dom))
    with pytest.raises(RuntimeError, match="Neighbor list overflow"):
        sim.run(5)
    assert not nl.status_pending
    nl.check_status()  # nothing left to raise


def test_rebuild_is_deterministic(gpu):
    """The re-sorted layout depends only on positions: two builds agree bit for bit."""
    import taichimps_gb300 as G
    from taichimps_gb300.packing import config1
    p = config1(seed=4)
    outs = []
    for _ in range(2):
        dom = G.Domain(boxlo=[0.0] * 3, boxhi=[p["L"]] * 3)
        atom = G.AtomSystem(max_atoms=len(p["x"]))
        atom.add_particles(x=p["x"], radius=p["radius"], density=2.5)
        nl = G.NeighborList(domain=dom, skin=0.1, max_atoms=len(p["x"]), max_neighbors_per_atom=32)
        nl.build(atom)
        nbr, nnb = nl.full_rows()  # entries past a row's length are unspecified
        outs.append((nbr, nnb, atom.buffers.uid.cpu().numpy().copy()))
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
