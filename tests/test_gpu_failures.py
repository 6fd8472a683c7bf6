"""
Failure detection without a GPU fault: a non-finite position is reported as an
exception on the host, never as a hang or a device trap.

The reference's skin check (neighbor.py:242-245) compares |x - x0|^2 > trigger,
which a NaN never satisfies, so a blown-up run there keeps stepping on NaN
positions.  Here the skin checks (fused step A, per-hook tmps_skin_check) treat a
non-finite displacement as a crossing, the rebuild that follows bins the atom,
finds it non-finite (TMPS_STATUS_NONFINITE) and NeighborList.build raises.  The
faults are made on the host: a NaN written into one atom's state between runs.
"""

import math

import numpy as np
import pytest

from _twin import dense_packing, make_twin

pytestmark = pytest.mark.gpu


def _system(oracle, precision, fused=True):
    rng = np.random.default_rng(41)
    x, r = dense_packing(rng, 216, 6.2, 0.48, 0.56)
    v = rng.normal(scale=0.05, size=x.shape)
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap="x")
    sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [6.2] * 3, v=v, pair="hertz/history", dt=5e-5,
                       cundall=(0.7, 0.7), deform=deform)
    sim.precision = precision
    sim.fused = fused
    return sim


@pytest.mark.parametrize("field", ["x", "v"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_state_raises_through_the_fused_step(gpu, oracle, precision, field):
    """A NaN position (or a NaN velocity, which the next drift carries into the position) in the middle of
    a fused run: the step's skin check forces the rebuild and the build raises."""
    sim = _system(oracle, precision)
    sim.run(10)
    assert sim.last_engine is not None
    sim.run_pre = False  # continue without the setup build, so the fused step itself meets the NaN
    b = sim.atom.buffers
    rec = b.xr if field == "x" else b.vm  # (x, radius) / (v, mass) records, internal order
    rec[17, 1] = math.nan
    with pytest.raises(RuntimeError, match="non-finite"):
        sim.run(10)


def test_nonfinite_position_raises_through_the_per_hook_path(gpu, oracle):
    sim = _system(oracle, "fp64", fused=False)
    sim.run(5)
    assert sim.last_engine is None
    sim.run_pre = False
    sim.atom.buffers.xr[3, 2] = math.inf
    with pytest.raises(RuntimeError, match="non-finite"):
        sim.run(5)


def test_finite_run_is_unaffected(gpu, oracle):
    """The crossing test !(q <= trigger) takes the same decisions as q > trigger for finite values: a
    clean run rebuilds exactly when the oracle does."""
    rng = np.random.default_rng(42)
    x, r = dense_packing(rng, 216, 6.2, 0.48, 0.56)
    v = rng.normal(scale=1.0, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [6.2] * 3, v=v, pair="hertz/history", dt=5e-5, skin=0.004)
    sim.run(80)
    osim.run(80)
    assert sim.neighbor.build_count == osim.neighbor.build_count > 3
