"""
fix deform/pressure's volume style (one_from_one, one_from_two, two_from_one,
vol/balance/p) and box style (volume, pressure) on the device -- the
reference runs them on its host path (deform_pressure.py:858-1001) -- against
the oracle's restatement of that path, through the fused step and the per-hook
path: the box to 1e-12, the state to 1e-10.
"""

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin, oracle_state, rel_err

pytestmark = pytest.mark.gpu

P = lambda: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-2}
CASES = {
    "volume_one_from_one": dict(axes={"x": {"style": "erate", "rate": -0.5}, "y": {"style": "volume"}}),
    "volume_two_from_one": dict(axes={"x": {"style": "volume"}, "y": {"style": "volume"},
                                      "z": {"style": "erate", "rate": -0.5}}),
    "volume_one_from_two": dict(axes={"x": P(), "y": {"style": "volume"}, "z": {"style": "erate", "rate": -0.5}}),
    "vol_balance_p": dict(axes={"x": {"style": "volume"}, "y": {"style": "volume"},
                                "z": {"style": "erate", "rate": -0.5}}, vol_balance_p=True, max_rate=0.2),
    "box_volume": dict(axes={"x": {"style": "erate", "rate": -0.5}, "y": P()}, box={"style": "volume"}),
    "box_pressure": dict(axes={"x": {"style": "erate", "rate": 0.3}},
                         box={"style": "pressure", "ptarget": 1.0, "pgain": 1e-2}, max_rate=0.5),
}


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("case", list(CASES))
def test_volume_and_box_styles_match_oracle(gpu, oracle, case, fused):
    rng = np.random.default_rng(41)
    box = 8.0
    x, r = dense_packing(rng, 512, box, 0.48, 0.56)
    deform = dict(remap="x", **CASES[case])
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7), deform=deform)
    sim.fused = fused
    steps = 150
    sim.run(steps)
    osim.run(steps)
    sim.domain.pull()
    prd = np.array(sim.domain.boxhi) - np.array(sim.domain.boxlo)
    assert np.abs(osim.domain.prd - box).max() > 1e-4          # the box did move
    np.testing.assert_allclose(prd, osim.domain.prd, rtol=1e-12, atol=0)
    np.testing.assert_allclose(sim.domain.boxlo, osim.domain.boxlo, rtol=0, atol=1e-12 * box)
    if case.startswith("volume") or case == "vol_balance_p" or case == "box_volume":
        assert float(np.prod(prd)) == pytest.approx(box ** 3, rel=1e-12)   # volume held
    g, o = gpu_state(sim), oracle_state(osim)
    for k in ("x", "v", "f", "torque"):
        assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))


def test_volume_style_mixed_form(gpu, oracle):
    """The mixed form carries the same post-pass: box within 1e-9, state within the mixed tolerances."""
    rng = np.random.default_rng(43)
    box = 8.0
    x, r = dense_packing(rng, 512, box, 0.48, 0.56)
    deform = dict(remap="x", **CASES["volume_one_from_two"])
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7), deform=deform)
    sim.precision = "mixed"
    sim.run(150)
    osim.run(150)
    sim.domain.pull()
    prd = np.array(sim.domain.boxhi) - np.array(sim.domain.boxlo)
    np.testing.assert_allclose(prd, osim.domain.prd, rtol=1e-9)
    g, o = gpu_state(sim), oracle_state(osim)
    assert rel_err(g["f"], o["f"]) < 5e-4
