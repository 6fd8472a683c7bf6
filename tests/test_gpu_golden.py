"""
The reference's own known answers, run through the GPU path's drop-in API the
way the reference's tests run them.  Inputs and expected values come from
tests/golden/known_answers.json, which make_known_answers.py reads out of the
reference's test files (each case cites its file:line).
"""

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())["cases"]


def _system(G, case, max_atoms=10):
    d = case["domain"]
    dom = G.Domain(boxlo=d["boxlo"], boxhi=d["boxhi"], boundary=d["boundary"])
    atom = G.AtomSystem(max_atoms=max_atoms)
    p = case["particles"]
    atom.add_particles(x=p["x"], v=p.get("v"), radius=p["radius"], density=p["density"], tag=p.get("tag"),
                       atom_type=p.get("atom_type", 1))
    return dom, atom


def test_hooke_known_answer(gpu):
    """tests/test_hooke.py: F = 4288.790204786391 (LAMMPS-verified), rtol 1e-12."""
    import taichimps_gb300 as G
    c = CASES["hooke_normal_contact"]
    dom, atom = _system(G, c)
    nl = G.NeighborList(domain=dom, skin=c["skin"], max_atoms=10, max_neighbors=10)
    nl.build(atom)
    hist = G.ContactHistory(max_atoms=10, max_neighbors=10)
    pair = G.GranHooke(domain=dom, **c["pair"])
    pair.compute(atom, nl, hist, dt=c["dt"])
    f = atom.f.to_numpy()
    np.testing.assert_allclose(f[0], [c["expected_fx"][0], 0.0, 0.0], rtol=c["rtol"])
    np.testing.assert_allclose(f[1], [c["expected_fx"][1], 0.0, 0.0], rtol=c["rtol"])


def test_pbc_wrap_known_answer(gpu):
    """tests/test_domain_neighbor.py: 10.5 -> 0.5, -0.2 -> 9.8 in a [0, 10) periodic box."""
    import taichimps_gb300 as G
    c = CASES["pbc_wrap"]
    dom, atom = _system(G, c)
    dom.pbc(atom)
    x = atom.x.to_numpy()[0]
    assert (0.0 <= x).all() and (x < 10.0).all()
    for k, v in c["expected"].items():
        assert np.isclose(x[int(k)], v), (k, x)


def test_neighbor_list_known_answer(gpu):
    """tests/test_domain_neighbor.py: atom 0's only neighbor is atom 1 (1.5 < 2.2 < 5.0)."""
    import taichimps_gb300 as G
    c = CASES["neighbor_list"]
    dom, atom = _system(G, c)
    nl = G.NeighborList(domain=dom, skin=c["skin"], max_atoms=10, max_neighbors=10)
    nl.build(atom)
    nn = nl.num_neighbors.to_numpy()
    assert nn[0] == len(c["neighbors_of_0"])
    assert list(nl.neighbors.to_numpy()[0, :nn[0]]) == c["neighbors_of_0"]


def test_skin_trigger_known_answer(gpu):
    """tests/test_domain_neighbor.py: a move of 0.08 < skin/2 keeps the list, 0.12 > skin/2 rebuilds."""
    import taichimps_gb300 as G
    c = CASES["skin_trigger"]
    dom, atom = _system(G, c)
    nl = G.NeighborList(domain=dom, skin=c["skin"], max_atoms=10, max_neighbors=10)
    assert nl.check_and_build(atom, timestep=0) is True
    assert nl.check_and_build(atom, timestep=1) is False
    for t, (pos, expect) in enumerate(zip(c["moves"], c["rebuild_expected"]), start=2):
        atom.x[0] = pos
        assert nl.check_and_build(atom, timestep=t) is expect
    assert nl.build_count == 2
