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
