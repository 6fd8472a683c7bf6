"""
NeighborList(slots="auto"): the full-list slot count follows the longest row
of each build (shrunk to fit, grown and rebuilt on an overflow) and the
contact history is carried across every change.  A run with auto slots is
bit-identical to one with a fixed cap: the per-hook path, the fused step in
both forms, with rebuilds.
"""

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin

pytestmark = pytest.mark.gpu


def _twin_run(oracle, precision, fused, slots, start=None, steps=200):
    rng = np.random.default_rng(13)
    x, r = dense_packing(rng, 512, 8.0, 0.48, 0.58)
    v = rng.normal(scale=2.0, size=x.shape)
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap="x")
    sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [8.0] * 3, v=v, pair="hertz/history", dt=5e-5, skin=0.02,
                       cundall=(0.7, 0.7), deform=deform)
    import taichimps_gb300 as G
    nl = G.NeighborList(domain=sim.domain, skin=0.02, max_atoms=len(x), max_neighbors_per_atom=32, slots=slots)
    if start is not None:
        nl.slots = nl.prev_slots = start
    sim.neighbor = nl
    sim.precision = precision
    sim.fused = fused
    sim.run(steps)
    return sim


@pytest.mark.parametrize("precision,fused", [("fp64", False), ("fp64", True), ("mixed", True)])
def test_auto_slots_bit_identical(gpu, oracle, precision, fused):
    ref = _twin_run(oracle, precision, fused, 64)
    auto = _twin_run(oracle, precision, fused, "auto")
    assert auto.neighbor.build_count > 2
    assert auto.neighbor.slots < 64                     # shrunk to fit the rows
    assert int(auto.neighbor.nnb.max()) <= auto.neighbor.slots
    g, h = gpu_state(ref), gpu_state(auto)
    for k in ("x", "v", "omega", "f", "torque"):
        np.testing.assert_array_equal(g[k], h[k], err_msg=k)


def test_auto_slots_grow_on_overflow(gpu, oracle):
    """Starting from 4 slots, the first build overflows, grows and rebuilds; the run is the same."""
    ref = _twin_run(oracle, "fp64", True, 64)
    auto = _twin_run(oracle, "fp64", True, "auto", start=4)
    assert auto.neighbor.slots > 4
    g, h = gpu_state(ref), gpu_state(auto)
    for k in ("x", "v", "omega", "f", "torque"):
        np.testing.assert_array_equal(g[k], h[k], err_msg=k)
