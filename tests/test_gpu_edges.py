"""
Edge sizes through the fused step and the batched runs: systems of one, two
and a few atoms (a count below, at and just past one 32-atom group), a pair
whose contact crosses the periodic boundary, an atom that wraps the box, and
a batch whose instances include single atoms.  Each against the oracle (FP64
to 1e-10; mixed within the fused-step tolerances) or, for the batch, bit for
bit against the same instances run one at a time.
"""

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin, oracle_state, rel_err

pytestmark = pytest.mark.gpu

MIXED_F = 5e-4
MIXED_V = 5e-4
MIXED_X = 1e-9


def _deform(max_rate=1e-2):
    return dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                max_rate=max_rate, remap="x")


def _compare(sim, osim, precision, box):
    g, o = gpu_state(sim), oracle_state(osim)
    if precision == "fp64":
        for k in ("x", "v", "omega", "f", "torque"):
            assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
        np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-12)
    else:
        assert np.abs(g["x"] - o["x"]).max() <= MIXED_X * box
        assert rel_err(g["v"], o["v"]) < MIXED_V, rel_err(g["v"], o["v"])
        assert rel_err(g["f"], o["f"]) < MIXED_F, rel_err(g["f"], o["f"])
        np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-9)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_single_atom_wraps_the_box(gpu, oracle, precision):
    """One atom, no partner: it crosses the periodic boundary and forces list rebuilds; the servo
    sees only its kinetic pressure."""
    box = 4.0
    x = np.array([[3.95, 0.5, 2.0]])
    v = np.array([[90.0, -40.0, 5.0]])
    sim, osim = make_twin(oracle, x, np.array([0.5]), 2.5, [0.0] * 3, [box] * 3, v=v, pair="hertz/history",
                          dt=5e-5, deform=_deform())
    sim.precision = precision
    sim.run(60)
    osim.run(60)
    assert sim.neighbor.build_count > 2
    assert 0.0 <= sim.atom.x.to_numpy()[0, 0] < sim.domain.prd[0]
    _compare(sim, osim, precision, box)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pair_across_periodic_boundary(gpu, oracle, precision):
    """Two atoms whose only contact is through the periodic image (shear history built up while
    they slide past each other)."""
    box = 4.0
    x = np.array([[0.1, 1.0, 1.0], [3.7, 1.05, 1.0]])
    v = np.array([[-1.0, 3.0, 0.0], [1.0, -3.0, 0.5]])
    sim, osim = make_twin(oracle, x, np.array([0.2, 0.21]), 2.5, [0.0] * 3, [box] * 3, v=v,
                          pair="hertz/history", dt=5e-5, deform=_deform())
    sim.precision = precision
    sim.run(80)
    osim.run(80)
    assert np.abs(sim.atom.f.to_numpy()[:2]).max() > 0.0
    _compare(sim, osim, precision, box)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [2, 31, 32, 33])
def test_few_atoms_in_contact(gpu, oracle, precision, n):
    """Atom counts below, at and just past one 32-atom group, all in contact."""
    rng = np.random.default_rng(60 + n)
    side = int(np.ceil(n ** (1.0 / 3.0)))
    box = 1.0 * side
    x, r = dense_packing(rng, n, box, 0.48, 0.56)
    v = rng.normal(scale=0.5, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, v=v, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7), deform=_deform())
    sim.precision = precision
    sim.run(50)
    osim.run(50)
    _compare(sim, osim, precision, box)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_with_single_atom_instances(gpu, oracle, precision):
    """A batch whose instances include one-atom and two-atom systems beside a packed one: each
    instance bit for bit as when run on its own with the batch's launch shape."""
    import taichimps_gb300 as G

    def build():
        rng = np.random.default_rng(77)
        out = []
        xp, rp = dense_packing(rng, 64, 4.0, 0.48, 0.56)
        specs = [(np.array([[3.9, 1.0, 1.0]]), np.array([0.5]), np.array([[50.0, 0.0, 0.0]]), 4.0),
                 (xp, rp, rng.normal(scale=0.5, size=xp.shape), 4.0),
                 (np.array([[0.1, 1.0, 1.0], [3.7, 1.05, 1.0]]), np.array([0.2, 0.21]),
                  np.array([[-1.0, 3.0, 0.0], [1.0, -3.0, 0.5]]), 4.0),
                 (np.array([[1.0, 1.0, 1.0]]), np.array([0.3]), np.array([[0.0, 0.0, 0.0]]), 3.0)]
        for x, r, v, box in specs:
            sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, v=v, pair="hertz/history", dt=5e-5,
                               cundall=(0.7, 0.7), deform=_deform())
            sim.precision = precision
            out.append(sim)
        return out

    batch, single = build(), build()
    eng = G.BatchedEngine(batch, precision=precision, chunk=16)
    eng.run(48)
    for sb, ss in zip(batch, single):
        ss.launch_shape = eng.launch_shape
        ss.run(48)
        gb, gs = gpu_state(sb), gpu_state(ss)
        for k in ("x", "v", "omega", "f", "torque"):
            np.testing.assert_array_equal(gb[k], gs[k])
        np.testing.assert_array_equal(sb.domain.prd, ss.domain.prd)
        assert sb.neighbor.build_count == ss.neighbor.build_count
