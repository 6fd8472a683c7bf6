"""
Batched runs (taichimps_gb300/ensemble.py): instances of uneven size, each with
its own box, coefficients and servo, advanced together, give bit-identical
results to running each instance on its own -- including instances that
rebuild their lists at different steps.
"""

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin, rel_err, oracle_state

pytestmark = pytest.mark.gpu


def _instances(oracle, seed, moving):
    """Uneven systems: sizes, boxes, stiffness and friction differ; some move fast (skin rebuilds)."""
    import taichimps_gb300 as G
    rng = np.random.default_rng(seed)
    specs = [(64, 5.0), (216, 7.0), (125, 6.0), (343, 8.2), (27, 4.0), (512, 9.0)]
    out = []
    for k, (n, box) in enumerate(specs):
        x, r = dense_packing(rng, n, box, 0.45, 0.56)
        v = rng.normal(scale=(8.0 if (moving and k % 2) else 0.05), size=x.shape)
        kn = float(10 ** rng.uniform(4, 6))
        xmu = float(rng.uniform(0.1, 0.8))
        deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"},
                      couple="xyz", max_rate=1e-1, remap="x")
        sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, v=v, pair="hertz/history", dt=5e-5,
                              cundall=(0.7, 0.7), deform=deform)
        # own coefficients per instance (gran/hertz/history kn, kt = 2/7 kn, xmu)
        for p in (sim.pair_style.params, osim.pair.P):
            p.kn, p.kt = kn, kn * 2.0 / 7.0
        sim.pair_style.params.xmu = xmu
        osim.pair.P.xmu = xmu
        out.append((sim, osim))
    return out


def _assert_same(pairs_a, pairs_b):
    for (sb, _), (ss, _) in zip(pairs_a, pairs_b):
        assert sb.timestep == ss.timestep
        gb, gs = gpu_state(sb), gpu_state(ss)
        for k in ("x", "v", "omega", "f", "torque"):
            np.testing.assert_array_equal(gb[k], gs[k])
        np.testing.assert_array_equal(sb.domain.prd, ss.domain.prd)
        assert sb.neighbor.build_count == ss.neighbor.build_count


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batched_matches_single_runs(gpu, oracle, precision):
    """The tuned launch shape: every instance as its own single run of that shape."""
    import taichimps_gb300 as G
    batch = _instances(oracle, 51, moving=True)
    single = _instances(oracle, 51, moving=True)
    for sim, _ in batch + single:
        sim.precision = precision
    eng = G.BatchedEngine([s for s, _ in batch], precision=precision, chunk=16)
    eng.run(60)
    assert eng.rebuilds > 0 and eng.graph_replays > 0
    assert eng.tuning is not None and eng.launch_shape == eng.tuning["launch_shape"]
    for ss, _ in single:
        ss.launch_shape = eng.launch_shape
        ss.run(60)
        assert ss.timestep == 60
    _assert_same(batch, single)


@pytest.mark.parametrize("shape", [(1, 1), (4, 16), (32, 2)])
def test_fixed_shapes_match_single_runs(gpu, oracle, shape):
    import taichimps_gb300 as G
    batch = _instances(oracle, 53, moving=True)
    single = _instances(oracle, 53, moving=True)
    for sim, _ in batch + single:
        sim.precision = "mixed"
    G.BatchedEngine([s for s, _ in batch], precision="mixed", chunk=16, launch_shape=shape).run(40)
    for ss, _ in single:
        ss.launch_shape = shape
        ss.run(40)
    _assert_same(batch, single)


def test_tuning_leaves_the_run_untouched(gpu, oracle):
    """The tuner's trial launches write only copies: a tuned run equals an untuned run of the
    shape it picked, bit for bit."""
    import taichimps_gb300 as G
    tuned = _instances(oracle, 54, moving=True)
    fixed = _instances(oracle, 54, moving=True)
    eng = G.BatchedEngine([s for s, _ in tuned], precision="mixed", chunk=16)
    eng.run(40)
    G.BatchedEngine([s for s, _ in fixed], precision="mixed", chunk=16, launch_shape=eng.launch_shape).run(40)
    _assert_same(tuned, fixed)


def test_batched_matches_oracle(gpu, oracle):
    """FP64 batched run of instances with their own kn and xmu, against the oracle per instance."""
    import taichimps_gb300 as G
    pairs = _instances(oracle, 52, moving=False)
    for sim, _ in pairs:
        sim.precision = "fp64"
    G.BatchedEngine([s for s, _ in pairs], precision="fp64", chunk=16).run(40)
    for sim, osim in pairs:
        osim.run(40)
        g, o = gpu_state(sim), oracle_state(osim)
        for k in ("x", "v", "f"):
            assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
        np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-12)
