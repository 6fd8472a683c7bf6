"""Computes on the GPU path against the oracle: contact/atom (coordination number)."""

import numpy as np
import pytest

from _twin import dense_packing, make_twin

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("boundary", [("p", "p", "p"), ("f", "f", "p")])
def test_contact_count_matches_oracle(gpu, oracle, boundary):
    """ComputeContactAtom (computes/contact_atom.py:15-63): integer counts, bit-exact, insertion order."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(31)
    x, r = dense_packing(rng, 512, 8.0, 0.48, 0.58)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [8.0] * 3, boundary=boundary, pair="hertz/history")
    sim.neighbor.build(sim.atom)
    osim.neighbor.build(osim.atoms)
    got = G.ComputeContactAtom(max_atoms=512).compute(sim.atom, sim.domain, sim.neighbor)
    want = osim.neighbor.contact_count(osim.atoms)
    assert want.sum() > 0
    np.testing.assert_array_equal(got, want)
    assert G.ComputeContactAtom.reduce(got, "ave") == pytest.approx(want.mean())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_contact_count_after_fused_run(gpu, oracle, precision):
    """After a fused run the counts from the device state equal the oracle's after the same steps."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(32)
    x, r = dense_packing(rng, 343, 7.0, 0.5, 0.58)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.0] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7))
    sim.precision = precision
    sim.run(40)
    osim.run(40)
    got = G.ComputeContactAtom(max_atoms=343).compute(sim.atom, sim.domain, sim.neighbor)
    want = osim.neighbor.contact_count(osim.atoms)
    assert want.sum() > 0
    np.testing.assert_array_equal(got, want)
