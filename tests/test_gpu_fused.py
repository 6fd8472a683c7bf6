"""
The fused step (engine.py): FP64 form against the per-hook path and the oracle,
and the mixed form against the oracle with its error stated as a tolerance.

Mixed-form tolerances: the contact arithmetic is FP32, so the overlap
delta = radsum - r carries an absolute error of ~1e-7 (one FP32 ulp of r ~ 1);
at the overlaps used here (~0.02-0.1) forces are good to ~1e-5 relative.
"""

import numpy as np
import pytest

from _twin import dense_packing, gpu_state, make_twin, oracle_state, rel_err

pytestmark = pytest.mark.gpu

MIXED_F = 5e-4     # forces / torques, max-abs normalised
MIXED_V = 5e-4     # velocities after the run
MIXED_X = 1e-9     # positions (relative to the box)
MIXED_P = 1e-6     # pressure tensor driving the servo (the mixed form's accuracy gate; measured 1e-8 .. 6e-8)
MIXED_Q = 3e-6     # deviatoric stress q = p_zz - (p_xx + p_yy)/2, a difference of pressures (measured 8e-7)


def _servo_twin(oracle, precision, n=512, box=8.2, steps=60, seed=21, fused=True, remap="x", path="auto"):
    rng = np.random.default_rng(seed)
    x, r = dense_packing(rng, n, box, 0.48, 0.56)
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap=remap)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [box] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7), deform=deform)
    sim.precision = precision
    sim.fused = fused
    sim.contact_path = path
    sim.run(steps)
    osim.run(steps)
    return sim, osim


@pytest.mark.parametrize("path", ["screened", "rows"])
def test_fused_fp64_matches_per_hook_and_oracle(gpu, oracle, path):
    sim_f, osim = _servo_twin(oracle, "fp64", fused=True, path=path)
    assert sim_f.last_engine.rows == (path == "rows")
    sim_h, _ = _servo_twin(oracle, "fp64", fused=False)
    assert sim_f.last_engine is not None and sim_h.last_engine is None
    gf, gh, o = gpu_state(sim_f), gpu_state(sim_h), oracle_state(osim)
    for k in ("x", "v", "omega", "f", "torque"):
        assert rel_err(gf[k], o[k]) < 1e-10, (k, rel_err(gf[k], o[k]))
        assert rel_err(gf[k], gh[k]) < 1e-10, (k, rel_err(gf[k], gh[k]))
    np.testing.assert_allclose(sim_f.domain.prd, osim.domain.prd, rtol=1e-13)
    assert rel_err(sim_f.fixes[-1].last_pressure(), osim.last_pressure) < 1e-10
    assert sim_f.timestep == osim.timestep == 60


@pytest.mark.parametrize("path", ["screened", "rows"])
def test_mixed_matches_oracle_within_stated_error(gpu, oracle, path):
    sim, osim = _servo_twin(oracle, "mixed", path=path)
    assert sim.last_engine.rows == (path == "rows")
    assert sim.last_engine.mixed
    g, o = gpu_state(sim), oracle_state(osim)
    assert np.abs(o["f"]).max() > 0
    L = osim.domain.prd.max()
    assert np.abs(g["x"] - o["x"]).max() / L < MIXED_X, np.abs(g["x"] - o["x"]).max() / L
    assert rel_err(g["v"], o["v"]) < MIXED_V, rel_err(g["v"], o["v"])
    assert rel_err(g["f"], o["f"]) < MIXED_F, rel_err(g["f"], o["f"])
    assert rel_err(g["torque"], o["torque"]) < MIXED_F, rel_err(g["torque"], o["torque"])
    ep = rel_err(sim.fixes[-1].last_pressure(), osim.last_pressure)
    print(f"mixed vs oracle after 60 servo steps: pressure {ep:.2e}, f {rel_err(g['f'], o['f']):.2e}")
    assert ep < MIXED_P, ep
    np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_rebuild_every_step(gpu, oracle, precision):
    """check no: every step aborts the queued launches and rebuilds on the host."""
    rng = np.random.default_rng(11)
    x, r = dense_packing(rng, 343, 7.0, 0.5, 0.56)
    v = rng.normal(scale=0.05, size=x.shape)
    w = rng.normal(scale=0.5, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.0] * 3, v=v, w=w, pair="granular/mindlin", dt=5e-5)
    sim.precision = precision
    sim.neighbor.check = False
    osim.neighbor.check = False
    sim.run(12)
    osim.run(12)
    assert sim.neighbor.build_count == osim.neighbor.build_count == 13
    g, o = gpu_state(sim), oracle_state(osim)
    tol = 1e-10 if precision == "fp64" else MIXED_V
    assert rel_err(g["v"], o["v"]) < tol, rel_err(g["v"], o["v"])
    assert rel_err(g["f"], o["f"]) < (1e-9 if precision == "fp64" else MIXED_F)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_skin_triggered_rebuilds(gpu, oracle, precision):
    """Fast particles: the skin check fires every few steps inside queued chunks."""
    rng = np.random.default_rng(5)
    x, r = dense_packing(rng, 216, 7.5, 0.45, 0.5)
    v = rng.normal(scale=20.0, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.5] * 3, v=v, pair="hooke/history", dt=2e-4,
                          skin=0.1)
    sim.precision = precision
    sim.run(80)
    osim.run(80)
    assert osim.neighbor.build_count > 5
    assert sim.neighbor.build_count == osim.neighbor.build_count
    g, o = gpu_state(sim), oracle_state(osim)
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert rel_err(g["x"], o["x"]) < tol, rel_err(g["x"], o["x"])


def test_fused_second_run_continues(gpu, oracle):
    """Two run() calls: the setup evaluation between them (shearupdate off) as in the reference."""
    rng = np.random.default_rng(8)
    x, r = dense_packing(rng, 216, 6.2, 0.5, 0.56)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [6.2] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7))
    for _ in range(2):
        sim.run(15)
        osim.run(15)
    g, o = gpu_state(sim), oracle_state(osim)
    assert sim.timestep == 30
    assert rel_err(g["v"], o["v"]) < 1e-10 and rel_err(g["f"], o["f"]) < 1e-9


@pytest.mark.parametrize("path", ["screened", "rows"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_eager_launches(gpu, oracle, precision, path):
    """Chunks replayed as CUDA graphs give bit-identical results to launching step by step,
    across skin-triggered rebuilds (which force a new capture)."""
    rng = np.random.default_rng(9)
    x, r = dense_packing(rng, 216, 7.5, 0.45, 0.5)
    v = rng.normal(scale=10.0, size=x.shape)
    states = []
    for graphs in (True, False):
        sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.5] * 3, v=v, pair="hertz/history", dt=2e-4,
                           cundall=(0.7, 0.7))
        sim.precision = precision
        from taichimps_gb300.engine import FusedEngine
        sim.setup_run(200)
        sim.init_simulation()
        eng = FusedEngine(sim, precision, chunk=32, graphs=graphs, contact_path=path)
        eng.capture_first = graphs  # every whole chunk a graph replay, the first after each rebuild too
        eng.begin()
        eng.run(200)
        eng.finish()
        if graphs:
            assert eng.graph_replays > 0 and eng.rebuilds > 0
        states.append(gpu_state(sim))
    for k in ("x", "v", "omega", "f", "torque"):
        np.testing.assert_array_equal(states[0][k], states[1][k])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_first_chunk_runs_without_capture(gpu, oracle, precision):
    """A chunk whose launch arguments are new runs as plain launches; the next chunk with the same
    arguments is captured and replayed.  Three chunks without a rebuild: two replays, and the same
    bits as capturing from the first chunk on."""
    from taichimps_gb300.engine import FusedEngine
    from taichimps_gb300.packing import make_packing_box
    p = make_packing_box(1000, 0.8, 1.2, 0.45, seed=5, vel_sigma=0.5)
    L = [float(v) for v in p["L"]]
    states = []
    for capture_first in (False, True):
        sim, _ = make_twin(oracle, p["x"], p["radius"], 2.5, [0.0] * 3, L, v=p["v"], pair="hertz/history",
                           dt=5e-5)
        sim.precision = precision
        sim.setup_run(24)
        sim.init_simulation()
        eng = FusedEngine(sim, precision, chunk=8)
        eng.capture_first = capture_first
        eng.begin()
        eng.run(24)
        eng.finish()
        assert eng.rebuilds == 0
        assert eng.graph_replays == (3 if capture_first else 2)
        states.append(gpu_state(sim))
    for k in ("x", "v", "omega", "f", "torque"):
        np.testing.assert_array_equal(states[0][k], states[1][k])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_contact_bound_culling_is_exact(gpu, oracle, precision):
    """Skipping 32-atom groups that the gap bound rules out changes no bit of the
    result, and the culled run still matches the oracle.  A loose packing with
    moving spheres and a compressing servo (remap x): groups are culled early,
    contacts form later."""
    from taichimps_gb300.engine import FusedEngine
    from taichimps_gb300.packing import make_packing
    p = make_packing(2000, 0.9, 1.1, 0.40, seed=3, jitter=0.05, vel_sigma=0.1)
    L = p["L"]
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap="x")
    steps = 300
    states, culled = [], []
    for cull in (True, False):
        sim, osim = make_twin(oracle, p["x"], p["radius"], 2.5, [0.0] * 3, [L] * 3, v=p["v"], pair="hertz/history",
                              dt=5e-5, cundall=(0.7, 0.7), deform=deform)
        sim.setup_run(steps)
        sim.init_simulation()
        eng = FusedEngine(sim, precision, chunk=32, cull=cull, contact_path="screened")
        eng.begin()
        eng.run(steps // 2)
        culled.append(eng.cull_stats())
        eng.run(steps - steps // 2)
        eng.finish()
        sim.domain.pull()
        states.append(gpu_state(sim))
        if cull:
            osim.run(steps)
            o = oracle_state(osim)
            assert np.abs(o["f"]).max() > 0
            g = states[0]
            if precision == "fp64":
                for k in ("x", "v", "f", "torque"):
                    assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
            else:
                assert np.abs(g["x"] - o["x"]).max() / L < MIXED_X
                assert rel_err(g["v"], o["v"]) < MIXED_V
                assert rel_err(g["f"], o["f"]) < MIXED_F
    assert culled[0][1] > 0, culled       # the bound did rule groups out
    assert culled[1][1] == 0
    for k in ("x", "v", "omega", "f", "torque"):
        np.testing.assert_array_equal(states[0][k], states[1][k])


def test_zero_force_kicks_left_out_exactly(gpu, oracle):
    """The FP64 update leaves out the half-kicks of atoms whose force and torque
    are exact zeros (C flag clear) and only turns a negative zero velocity
    component into +0, as adding the zero kick would: the run is bit for bit
    the one that kicks every atom (kick_all set on the device).  Negative zero
    components are written into contact-free atoms mid-run, after the first
    contact pass has cleared their flags."""
    from taichimps_gb300 import _device, _lib
    from taichimps_gb300.engine import FusedEngine
    from taichimps_gb300.packing import make_packing
    p = make_packing(2000, 0.9, 1.1, 0.40, seed=5, jitter=0.05, vel_sigma=0.1)
    L = p["L"]
    states = []
    for kick_all in (False, True):
        sim, _ = make_twin(oracle, p["x"], p["radius"], 2.5, [0.0] * 3, [L] * 3, v=p["v"], pair="hertz/history",
                           dt=5e-5, cundall=(0.7, 0.7), skin=0.3)
        sim.setup_run(80)
        sim.init_simulation()
        eng = FusedEngine(sim, "fp64", chunk=16, contact_path="screened")
        eng.begin()
        assert _device.pull_struct(eng._eng, _lib.Engine).kick_all == 0  # every 1/m, 1/I positive and finite
        if kick_all:
            e = _lib.Engine()
            e.kick_all = 1
            _device.push_fields(eng._eng, e, "kick_all", "kick_all")
        eng.run(40)
        vm, om = sim.atom._buf.vm, sim.atom._buf.om
        vm[::7, 0] = -0.0
        vm[3::11, 2] = -0.0
        om[5::13, 1] = -0.0
        eng.run(40)
        eng.finish()
        assert eng.rebuilds == 0  # a rebuild's prepare would reset kick_all
        states.append(gpu_state(sim))
    for k in ("x", "v", "omega", "f", "torque"):
        a, b = (np.ascontiguousarray(s[k]).view(np.int64) for s in states)
        np.testing.assert_array_equal(a, b, err_msg=k)
    for k in ("v", "omega"):
        z = states[0][k] == 0.0
        assert z.any() and not np.signbit(states[0][k][z]).any(), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pressure_record_each_step(gpu, oracle, precision):
    """record_pressure: every fused step writes the servo's pressure tensor to pinned host memory; the
    ring holds the last steps, the final row is the servo's own, and each row matches the oracle's
    pressure after that many steps."""
    rng = np.random.default_rng(4)
    x, r = dense_packing(rng, 343, 7.6, 0.48, 0.56)
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap="x")
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.6] * 3, pair="hertz/history", dt=5e-5,
                          cundall=(0.7, 0.7), deform=deform)
    sim.precision = precision
    fix = sim.fixes[-1]
    fix.record_pressure(8)
    sim.run(70)
    rows = fix.pressure_history(range(63, 71))
    np.testing.assert_array_equal(rows[-1], fix.last_pressure())
    assert np.isfinite(rows).all() and np.abs(rows).max() > 0
    tol = 1e-10 if precision == "fp64" else MIXED_P
    osim.run(62)
    errs = []
    for k, s in enumerate(range(63, 71)):
        osim.step()
        errs.append(rel_err(rows[k], osim.last_pressure))
        assert errs[-1] < tol, (s, errs[-1])
    print(f"{precision} pressure record vs oracle, steps 63-70: max {max(errs):.2e}")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_rolling_resistance(gpu, oracle, precision):
    """The triaxial configuration's contact (pair granular hertz/material, coeff_restitution, mindlin,
    rolling EPSD) through the fused step with Cundall and the servo, against the oracle; spinning
    spheres so the rolling torque and its history matter."""
    rng = np.random.default_rng(17)
    x, r = dense_packing(rng, 343, 7.2, 0.5, 0.57)
    w = rng.normal(scale=2.0, size=x.shape)
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-1, remap="x")
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.2] * 3, w=w, pair="granular/rolling", dt=5e-5,
                          cundall=(0.7, 0.7), deform=deform)
    sim.precision = precision
    sim.run(50)
    osim.run(50)
    assert sim.last_engine is not None
    assert np.abs(osim.history.rolling).max() > 0
    g, o = gpu_state(sim), oracle_state(osim)
    if precision == "fp64":
        for k in ("x", "v", "omega", "f", "torque"):
            assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
    else:
        assert rel_err(g["f"], o["f"]) < MIXED_F, rel_err(g["f"], o["f"])
        assert rel_err(g["torque"], o["torque"]) < MIXED_F, rel_err(g["torque"], o["torque"])
        assert rel_err(g["omega"], o["omega"]) < MIXED_V, rel_err(g["omega"], o["omega"])


@pytest.mark.parametrize("path", ["screened", "rows"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_partial_last_group_flags_and_no_spurious_rebuild(gpu, oracle, precision, path):
    """An atom count that is not a multiple of 32: the flag words set after a
    build carry no bit past the last atom (a set bit makes C clear that atom's
    force, so a bit past the end would write past the force arrays), and a
    packing at rest with a servo barely moving the box never trips the skin
    check (only the setup build)."""
    import torch
    from taichimps_gb300.engine import FusedEngine
    from taichimps_gb300.packing import make_packing_box
    n = 1363
    p = make_packing_box(n, 0.8, 1.2, 0.45, seed=17)
    L = [float(v) for v in p["L"]]
    deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
                  max_rate=1e-4, remap="x")
    sim, _ = make_twin(oracle, p["x"], p["radius"], 2.5, [0.0] * 3, L, pair="hertz/history", dt=5e-5,
                       deform=deform)
    sim.setup_run(40)
    sim.init_simulation()
    eng = FusedEngine(sim, precision, chunk=8, contact_path=path)
    eng.begin()
    ng = (n + 31) // 32
    words = eng.part[:4 * ng].view(torch.int32).cpu().numpy().view(np.uint32)
    assert words[-1] == (1 << (n % 32)) - 1, hex(words[-1])
    assert np.all(words[:-1] == 0xFFFFFFFF)
    if precision == "mixed":
        o0 = eng.o0.clone()
    eng.run(40)
    assert eng.rebuilds == 0
    if precision == "mixed":
        assert bool((eng.o0 == o0).all())
    words = eng.part[:4 * ng].view(torch.int32).cpu().numpy().view(np.uint32)
    assert (int(words[-1]) >> (n % 32)) == 0
    eng.finish()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_triaxial_loading_matches_oracle(gpu, oracle, precision):
    """The triaxial loading (pair granular with mindlin and rolling EPSD; x and y pressure-servoed at
    1.0, z strain-controlled at erate -1e-3, remap x) through the fused step: the deviatoric stress
    q = p_zz - (p_xx + p_yy)/2 of every step, the box and the coordination number after 120 steps
    against the oracle."""
    from taichimps_gb300 import ComputeContactAtom
    rng = np.random.default_rng(29)
    x, r = dense_packing(rng, 343, 7.2, 0.5, 0.56)
    deform = dict(axes={"x": {"style": "pressure", "ptarget": 1.0, "pgain": 0.1},
                        "y": {"style": "pressure", "ptarget": 1.0, "pgain": 0.1},
                        "z": {"style": "erate", "rate": -1e-3}}, max_rate=1e-2, remap="x")
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.2] * 3, pair="granular/rolling", dt=5e-5,
                          deform=deform)
    sim.precision = precision
    fix = sim.fixes[-1]
    fix.record_pressure(128)
    steps = 120
    sim.run(steps)
    rows = fix.pressure_history(range(1, steps + 1))
    q = rows[:, 2] - 0.5 * (rows[:, 0] + rows[:, 1])
    osim.setup(steps)
    oq = []
    for _ in range(steps):
        osim.step()
        P = osim.last_pressure
        oq.append(P[2] - 0.5 * (P[0] + P[1]))
    oq = np.array(oq)
    assert np.abs(oq).max() > 0
    tol = 1e-10 if precision == "fp64" else MIXED_Q
    eq = np.abs(q - oq).max() / np.abs(oq).max()
    print(f"{precision} triaxial q vs oracle over 120 steps: {eq:.2e}")
    assert eq < tol, eq
    sim.domain.pull()
    np.testing.assert_allclose(np.array(sim.domain.boxhi) - np.array(sim.domain.boxlo), osim.domain.prd,
                               rtol=1e-12 if precision == "fp64" else 1e-9)
    cn = ComputeContactAtom(max_atoms=len(x)).compute(sim.atom, sim.domain, sim.neighbor)
    ocn = osim.neighbor.contact_count(osim.atoms)
    if precision == "fp64":
        np.testing.assert_array_equal(cn, ocn)
    else:
        assert abs(cn.mean() - ocn.mean()) <= 0.02 * ocn.mean()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_launch_shape_changes_rounding_only(gpu, oracle, precision):
    """A non-default launch shape (more 32-atom groups per warp of A and C, fewer blocks) changes only
    the order of the virial sum: the run stays within the stated tolerances of the oracle, and two
    runs of the same shape are bit-identical."""
    runs = []
    for _ in range(2):
        rng = np.random.default_rng(23)
        x, r = dense_packing(rng, 1000, 10.0, 0.48, 0.56)
        deform = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"},
                      couple="xyz", max_rate=1e-1, remap="x")
        sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [10.0] * 3, pair="hertz/history", dt=5e-5,
                              cundall=(0.7, 0.7), deform=deform)
        sim.precision = precision
        sim.launch_shape = (2, 4)
        sim.run(60)
        eng = sim.last_engine
        assert eng.c_blocks == 2 and eng.a_blocks == 2
        runs.append((sim, osim))
    (sim, osim), (sim2, _) = runs
    g, g2 = gpu_state(sim), gpu_state(sim2)
    for k in ("x", "v", "omega", "f", "torque"):
        np.testing.assert_array_equal(g[k], g2[k])
    osim.run(60)
    o = oracle_state(osim)
    if precision == "fp64":
        for k in ("x", "v", "omega", "f", "torque"):
            assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
        np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-12)
    else:
        assert rel_err(g["f"], o["f"]) < MIXED_F
        assert rel_err(g["v"], o["v"]) < MIXED_V
        np.testing.assert_allclose(sim.domain.prd, osim.domain.prd, rtol=1e-9)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_neighbor_delay_every_check(gpu, oracle, precision):
    """neigh_modify delay 5 every 3 check yes through the fused step: a rebuild only once 5 steps have
    passed since the last one, only on every third step, and only when an atom moved more than half the
    skin (NeighborList.decide, neighbor.py:371-403).  The rebuild steps match the oracle's step by step
    (runs of 7 steps continuing one another), and so does the state."""
    rng = np.random.default_rng(57)
    x, r = dense_packing(rng, 343, 7.0, 0.5, 0.56)
    v = rng.normal(scale=0.8, size=x.shape)
    w = rng.normal(scale=2.0, size=x.shape)
    sim, osim = make_twin(oracle, x, r, 2.5, [0.0] * 3, [7.0] * 3, v=v, w=w, pair="hertz/history", dt=5e-5,
                          skin=0.004, cundall=(0.7, 0.7))
    sim.precision = precision
    for nl in (sim.neighbor, osim.neighbor):
        nl.delay, nl.every, nl.check = 5, 3, True
    builds, obuilds = [], []
    for seg in range(9):
        sim.run(7)
        if seg == 0:
            osim.run(7)
        else:  # the oracle's step() continues a run without the setup pass (run 7 pre no)
            for _ in range(7):
                osim.step()
        sim.run_pre = False
        builds.append((sim.neighbor.build_count, sim.neighbor.last_build_step))
        obuilds.append((osim.neighbor.build_count, osim.neighbor.last_build_step))
    assert builds == obuilds, (builds, obuilds)
    # rebuilds happened, all at steps that the delay and every rules allow
    assert builds[-1][0] >= 4
    assert all(b[1] % 3 == 0 for b in builds)
    g, o = gpu_state(sim), oracle_state(osim)
    if precision == "fp64":
        for k in ("x", "v", "omega", "f", "torque"):
            assert rel_err(g[k], o[k]) < 1e-10, (k, rel_err(g[k], o[k]))
    else:
        assert rel_err(g["v"], o["v"]) < MIXED_V, rel_err(g["v"], o["v"])
        assert rel_err(g["f"], o["f"]) < MIXED_F, rel_err(g["f"], o["f"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("pair", ["hertz/history", "granular/rolling"])
def test_rows_path_equals_screened_path(gpu, oracle, precision, pair):
    """C's per-atom-row path and its screened path sum each atom's contacts in slot order with the same
    per-contact code; without a servo the order of the virial partial sums feeds nothing back.  For
    gran/hertz/history the two runs (with rebuilds) are bit-identical.  The pair granular law has sums of
    two products whose multiply-add contraction the compiler may pick differently in the two kernels, so
    there the runs agree to rounding (FP64: 1e-12 after 40 steps; mixed: the mixed form's tolerances)."""
    import torch
    rng = np.random.default_rng(5)
    x, r = dense_packing(rng, 512, 8.2, 0.48, 0.56)
    v = rng.normal(scale=0.05, size=x.shape)
    w = rng.normal(scale=0.5, size=x.shape)
    states = []
    for path in ("screened", "rows"):
        sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [8.2] * 3, v=v, w=w, pair=pair, dt=5e-5,
                           cundall=(0.7, 0.7))
        sim.precision = precision
        sim.contact_path = path
        sim.run(40)
        assert sim.last_engine.rows == (path == "rows")
        st = gpu_state(sim)
        st["touch"] = sim.history.touch.cpu().numpy()
        st["shear"] = sim.history.shear.cpu().numpy()
        st["builds"] = sim.neighbor.build_count
        states.append(st)
    assert np.abs(states[0]["f"]).max() > 0 and np.count_nonzero(states[0]["touch"]) > 256
    assert states[0]["builds"] == states[1]["builds"]
    if pair == "hertz/history":
        for k in ("x", "v", "omega", "f", "torque", "touch"):
            np.testing.assert_array_equal(states[0][k], states[1][k])
        live = (states[0]["touch"][None, :] >> np.arange(states[0]["shear"].shape[1], dtype=np.int64)[:, None]) & 1
        for c in range(3):
            np.testing.assert_array_equal(states[0]["shear"][c][live == 1], states[1]["shear"][c][live == 1])
    else:
        tol = {"x": 1e-12, "v": 1e-12, "omega": 1e-12, "f": 1e-12, "torque": 1e-12} if precision == "fp64" else \
              {"x": MIXED_X, "v": MIXED_V, "omega": MIXED_V, "f": MIXED_F, "torque": MIXED_F}
        for k, t in tol.items():
            e = np.abs(states[0][k] - states[1][k]).max() / (8.2 if k == "x" else np.abs(states[0][k]).max())
            assert e < t, (k, e)


def test_auto_contact_path(gpu, oracle):
    """contact_path "auto": the per-atom-row path on a packing where most atoms overlap at the build, the
    screened path on a loose one."""
    from taichimps_gb300.packing import make_packing_box
    rng = np.random.default_rng(6)
    x, r = dense_packing(rng, 512, 8.2, 0.48, 0.56)
    sim, _ = make_twin(oracle, x, r, 2.5, [0.0] * 3, [8.2] * 3, pair="hertz/history", dt=5e-5)
    sim.precision = "mixed"
    sim.run(5)
    assert sim.last_engine.rows
    p = make_packing_box(1363, 0.8, 1.2, 0.45, seed=17)
    sim, _ = make_twin(oracle, p["x"], p["radius"], 2.5, [0.0] * 3, [float(v) for v in p["L"]],
                       pair="hertz/history", dt=5e-5)
    sim.precision = "mixed"
    sim.run(5)
    assert not sim.last_engine.rows
