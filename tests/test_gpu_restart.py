"""
Contact history through a restart (contact_history.py:155-214, restart.py:694-715):
touching_by_atom gives one entry per contact under its lower-index atom, the
restart writer's expansion gives LAMMPS' both-sided records, and load_restart
puts them back onto a fresh list at its first build.
"""

import numpy as np
import pytest

from _twin import dense_packing, make_twin

pytestmark = pytest.mark.gpu


def _both_sided(own, tags):
    """restart.py:694-715: each contact under both partners, the partner's copy negated."""
    index_of_tag = {int(t): i for i, t in enumerate(tags)}
    out = [[] for _ in own]
    for i, row in enumerate(own):
        for ptag, value in row:
            out[i].append((ptag, value))
            j = index_of_tag.get(ptag)
            if j is not None:
                out[j].append((int(tags[i]), -value))
    return out


def _fresh(oracle, sim, x, r):
    a = sim.atom
    n = a.nlocal
    s2, _ = make_twin(oracle, a.x.to_numpy()[:n], r, 2.5, [0.0] * 3, [7.0] * 3, v=a.v.to_numpy()[:n],
                      w=a.omega.to_numpy()[:n], pair="hertz/history", dt=5e-5, cundall=(0.7, 0.7))
    return s2


def test_restart_history_round_trip(gpu, oracle):
    rng = np.random.default_rng(44)
    x, r = dense_packing(rng, 343, 7.0, 0.5, 0.58)
    sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.0] * 3, pair="hertz/history", dt=5e-5,
                       cundall=(0.7, 0.7))
    sim.run(30)
    n = sim.atom.nlocal
    tags = sim.atom.tag.to_numpy()[:n]
    before = sim.history.contacts_by_tag(sim.neighbor)
    assert len(before) > 20 and max(np.abs(s).max() for s in before.values()) > 0
    own = sim.history.touching_by_atom(sim.neighbor, n)
    # one entry per contact, under the lower-index atom (tags follow insertion order here)
    assert sum(len(row) for row in own) * 2 == len(before)
    assert all(int(tags[i]) < ptag for i, row in enumerate(own) for ptag, _ in row)

    for records in (_both_sided(own, tags), own):   # LAMMPS' both-sided file, and one side only
        s2 = _fresh(oracle, sim, x, r)
        s2.history.load_restart([np.array([t for t, _ in row], dtype=np.int32) for row in records],
                                [np.array([v for _, v in row]).reshape(-1, 3) for row in records])
        s2.reneighbor_if_needed(force=True)
        after = s2.history.contacts_by_tag(s2.neighbor)
        assert set(after) == set(before)
        for key, val in before.items():
            np.testing.assert_array_equal(after[key], val)


def test_load_restart_rejects_overfull_atom(gpu):
    import taichimps_gb300 as G
    hist = G.ContactHistory(max_atoms=4, max_neighbors=2)
    with pytest.raises(ValueError, match="stored contacts but the history only has 2 slots"):
        hist.load_restart([np.array([2, 3, 4])], [np.zeros((3, 3))])


# ---------------------------------------------------------------- LAMMPS restart files


def _granular_twin(oracle, precision, pair, seed=45):
    rng = np.random.default_rng(seed)
    x, r = dense_packing(rng, 343, 7.0, 0.5, 0.58)
    v = rng.normal(scale=0.05, size=x.shape)
    w = rng.normal(scale=0.5, size=x.shape)
    sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.0] * 3, v=v, w=w, pair=pair, dt=5e-5,
                       cundall=(0.7, 0.7) if pair == "hertz/history" else None)
    sim.precision = precision
    return sim


def _sim_from_file(path, like, precision):
    """A Simulation rebuilt from a restart file (taichimps_gb300.restart.system_from_restart), with the
    neighbor settings and fixes of `like`."""
    import taichimps_gb300 as G
    from taichimps_gb300.restart import read_restart, system_from_restart
    data = read_restart(path)
    s = system_from_restart(data, max_neighbors=like.history.max_neighbors)
    dom = s["domain"]
    nl = G.NeighborList(domain=dom, skin=like.neighbor.skin, max_atoms=s["atom"].max_atoms,
                        max_neighbors_per_atom=like.neighbor.max_neighbors_per_atom)
    sim = G.Simulation(domain=dom, atom=s["atom"], neighbor=nl, history=s["history"], pair=s["pair"], dt=s["dt"],
                       precision=precision)
    sim.add_fix(G.FixNVESphere(domain=dom))
    for fx in like.fixes:
        if isinstance(fx, G.FixDampingCundall):
            sim.add_fix(G.FixDampingCundall(domain=dom, gamma_lin=fx.gamma_lin, gamma_ang=fx.gamma_ang))
    sim.timestep = s["timestep"]
    return sim, data


def _by_tag(sim):
    n = sim.atom.nlocal
    order = np.argsort(sim.atom.tag.to_numpy()[:n])
    return {k: getattr(sim.atom, k).to_numpy()[:n][order] for k in ("x", "v", "omega", "radius", "rmass")}


@pytest.mark.parametrize("pair", ["hertz/history", "granular/mindlin"])
def test_restart_file_holds_the_state(gpu, oracle, tmp_path, pair):
    """write_restart of a running system, read back: every array bit for bit, the pair style, and each
    touching contact under both of its atoms with the shear of that atom's side."""
    from taichimps_gb300.restart import read_restart, write_restart
    sim = _granular_twin(oracle, "fp64", pair)
    sim.run(40)
    f = tmp_path / "mid.restart"
    write_restart(f, sim.atom, sim.domain, timestep=sim.timestep, dt=sim.dt, history=sim.history,
                  pair=sim.pair_style, nlist=sim.neighbor)
    d = read_restart(f)
    n = sim.atom.nlocal
    assert d.timestep == 40 and d.natoms == n and d.dt == sim.dt
    for k in ("x", "v", "omega", "radius", "rmass"):
        np.testing.assert_array_equal(getattr(d, k), getattr(sim.atom, k).to_numpy()[:n])
    np.testing.assert_array_equal(d.tag, sim.atom.tag.to_numpy()[:n])
    assert d.pair_style == ("gran/hertz/history" if pair == "hertz/history" else "granular")
    live = sim.history.contacts_by_tag(sim.neighbor)
    assert len(live) > 20
    rows, ptag, vals = d.neigh_history()
    assert len(rows) == len(live)
    for r_, t, v in zip(rows, ptag, vals):
        np.testing.assert_array_equal(v, live[(int(d.tag[r_]), int(t))])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("pair", ["hertz/history", "granular/mindlin"])
def test_restart_continues_the_uninterrupted_run_bit_for_bit(gpu, oracle, tmp_path, precision, pair):
    """A run split by a restart file equals the same two runs without it (the reference's
    test_restart.py:294-316 split against `run N; run M`), bit for bit: the file keeps every double and
    the masses as stored, the history comes back on both copies of each contact, and the first build
    of the resumed run orders the atoms exactly as the continuing run's setup build does."""
    from taichimps_gb300.restart import write_restart
    half, total = 60, 140
    cont = _granular_twin(oracle, precision, pair)
    cont.run(half)
    cont.run(total - half)
    first = _granular_twin(oracle, precision, pair)
    first.run(half)
    f = tmp_path / "mid.restart"
    write_restart(f, first.atom, first.domain, timestep=first.timestep, dt=first.dt, history=first.history,
                  pair=first.pair_style, nlist=first.neighbor)
    second, _ = _sim_from_file(f, first, precision)
    second.run(total - half)
    assert second.timestep == cont.timestep == total
    a, b = _by_tag(cont), _by_tag(second)
    for k in ("x", "v", "omega"):
        np.testing.assert_array_equal(a[k], b[k])
    assert cont.history.contacts_by_tag(cont.neighbor).keys() == second.history.contacts_by_tag(second.neighbor).keys()


def test_periodic_restart_output(gpu, oracle, tmp_path):
    """restart 25 file.*: run(70) writes files at steps 25 and 50, each holding the state of a run
    stopped there; the segmented run ends where an unsegmented one does (FP64, bit for bit)."""
    from taichimps_gb300.restart import read_restart
    sim = _granular_twin(oracle, "fp64", "hertz/history")
    sim.set_restart(25, str(tmp_path / "state.*"))
    sim.run(70)
    assert sorted(p.name for p in tmp_path.iterdir()) == ["state.25", "state.50"]
    ref = _granular_twin(oracle, "fp64", "hertz/history")
    ref.run(70)
    a, b = _by_tag(ref), _by_tag(sim)
    for k in ("x", "v", "omega"):
        np.testing.assert_array_equal(a[k], b[k])
    at50 = _granular_twin(oracle, "fp64", "hertz/history")
    at50.run(50)
    d = read_restart(tmp_path / "state.50")
    assert d.timestep == 50
    n = at50.atom.nlocal
    np.testing.assert_array_equal(d.x, at50.atom.x.to_numpy()[:n])
    np.testing.assert_array_equal(d.v, at50.atom.v.to_numpy()[:n])
