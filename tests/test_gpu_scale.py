"""
Parity at the benchmark's scale, 1,000,000 spheres, against the oracle:

* the neighbor build -- grid, the cell of every atom and the pair set -- bit
  for bit, on the contact-free servo packing (make_packing, solid fraction
  0.45) and on the contact-dense one (a compressed 15,625-sphere cell tiled
  4 x 4 x 4, packing.dense_config2): the Morton grid of ~74k cells, the
  one-wave grids and the FP32 acceptance of the build far from the origin all
  run at this size only;
* the first step of the FP64 fused form on the dense packing: forces and
  torques within 1e-12, positions and velocities within 1e-13;
* the mixed form's mean pressure after 200 steps on the dense packing within
  1e-6 of the FP64 oracle (the accuracy gate of the mixed form), and the FP64
  form's within 1e-10.

The oracle runs on all host cores (OpenMP).
"""

import os

import numpy as np
import pytest

from _twin import rel_err

pytestmark = pytest.mark.gpu

KN = 2.0e5
PAIR = dict(kn=KN, kt=KN * 2.0 / 7.0, gamman=50.0, gammat=25.0, xmu=0.5, dampflag=1)
DEFORM = dict(axes={d: {"style": "pressure", "ptarget": 1.0, "pgain": 1e-3} for d in "xyz"}, couple="xyz",
              max_rate=1e-4, remap="x")
DT, SKIN = 5e-5, 0.1


@pytest.fixture(scope="module")
def all_cores(oracle):
    oracle.set_threads(os.cpu_count() or 1)
    yield oracle
    oracle.set_threads(1)


@pytest.fixture(scope="module")
def sparse1m(gpu):
    from taichimps_gb300.packing import config2
    return config2(seed=2, n=1_000_000)


@pytest.fixture(scope="module")
def dense1m(gpu):
    from taichimps_gb300.packing import dense_config2
    p = dense_config2(reps=(4, 4, 4))
    p["density"] = 2.5
    return p


def _box(p):
    L = np.broadcast_to(np.asarray(p["L"], dtype=np.float64), (3,))
    lo = np.asarray(p.get("lo", np.zeros(3)), dtype=np.float64)
    return [float(a) for a in lo], [float(a) for a in lo + L]


def _gpu_pair_keys(nl):
    """Every full-list entry as tag_lo << 32 | tag_hi, sorted (each pair appears twice)."""
    nbr, nnb = nl.full_rows()
    tag = nl._atom.buffers.tag.cpu().numpy().astype(np.int64)
    S = nbr.shape[0]
    k, p = np.nonzero(np.arange(S)[:, None] < nnb[None, :])
    a, b = tag[p], tag[nbr[k, p]]
    return np.sort((np.minimum(a, b) << 32) | np.maximum(a, b))


def _oracle_pair_keys(onl, tags):
    nn = np.asarray(onl.num_neighbors)
    nb = np.asarray(onl.neighbors)
    i, k = np.nonzero(np.arange(nb.shape[1])[None, :] < nn[:, None])
    a, b = tags[i].astype(np.int64), tags[nb[i, k]].astype(np.int64)
    return np.sort((np.minimum(a, b) << 32) | np.maximum(a, b))


@pytest.mark.parametrize("which", ["sparse", "dense"])
def test_neighbor_build_bit_exact_at_1m(all_cores, sparse1m, dense1m, which):
    import taichimps_gb300 as G
    O = all_cores
    p = sparse1m if which == "sparse" else dense1m
    n = len(p["x"])
    lo, hi = _box(p)
    dom = G.Domain(boxlo=lo, boxhi=hi)
    atom = G.AtomSystem(max_atoms=n)
    atom.add_particles(x=p["x"], radius=p["radius"], density=2.5)
    nl = G.NeighborList(domain=dom, skin=SKIN, max_atoms=n, max_neighbors_per_atom=32)
    nl.build(atom)
    odom = O.OracleDomain.make(lo, hi)
    oat = O.OracleAtoms(x=p["x"], radius=p["radius"], density=2.5)
    onl = O.OracleNeighbor(odom, skin=SKIN, max_neighbors=32)
    onl.build(oat)
    assert list(nl.grid_dim) == list(onl.grid_dim)
    assert int(np.prod(nl.grid_dim)) > 50_000
    cell_gpu = np.empty(n, dtype=np.int64)
    cell_gpu[atom.uid_host()] = nl.cell_of.cpu().numpy()
    np.testing.assert_array_equal(cell_gpu, onl.cell_of)
    g = _gpu_pair_keys(nl)
    # the full list holds every pair once from each side
    np.testing.assert_array_equal(g[0::2], g[1::2])
    o = _oracle_pair_keys(onl, oat.tag)
    assert len(o) > n // 2
    np.testing.assert_array_equal(g[0::2], o)


def _dense_pair(G, O, p, precision):
    n = len(p["x"])
    lo, hi = _box(p)
    dom = G.Domain(boxlo=lo, boxhi=hi)
    atom = G.AtomSystem(max_atoms=n)
    atom.add_particles(x=p["x"], radius=p["radius"], density=p["density"], v=p["v"])
    nl = G.NeighborList(domain=dom, skin=SKIN, max_atoms=n, max_neighbors_per_atom=32)
    hist = G.ContactHistory(max_atoms=n, max_neighbors=32)
    sim = G.Simulation(domain=dom, atom=atom, neighbor=nl, history=hist, pair=G.GranHertzHistory(domain=dom, **PAIR),
                       dt=DT, precision=precision)
    sim.add_fix(G.FixNVESphere(domain=dom))
    sim.add_fix(G.FixDampingCundall(domain=dom, gamma_lin=0.7, gamma_ang=0.7))
    sim.add_fix(G.FixDeformPressure(domain=dom, **DEFORM))
    odom = O.OracleDomain.make(lo, hi)
    oat = O.OracleAtoms(x=p["x"], radius=p["radius"], density=p["density"], v=p["v"])
    osim = O.OracleSim(odom, oat, O.OracleNeighbor(odom, skin=SKIN, max_neighbors=32), O.OracleHistory(32),
                       O.OraclePair("hertz/history", **PAIR), DT,
                       fixes=[O.OracleCundall(0.7, 0.7), O.OracleDeform(odom, **DEFORM)])
    return sim, osim


def test_dense_first_step_fp64_at_1m(all_cores, dense1m):
    import taichimps_gb300 as G
    sim, osim = _dense_pair(G, all_cores, dense1m, "fp64")
    sim.run(1)
    osim.run(1)
    n = sim.atom.nlocal
    g = {k: getattr(sim.atom, k).to_numpy()[:n] for k in ("x", "v", "f", "torque")}
    o = osim.atoms
    assert np.count_nonzero(np.abs(o.f).sum(1)) > 0.9 * n  # nearly every sphere is in contact
    assert rel_err(g["f"], o.f) < 1e-12, rel_err(g["f"], o.f)
    assert rel_err(g["torque"], o.torque) < 1e-12, rel_err(g["torque"], o.torque)
    assert rel_err(g["v"], o.v) < 1e-13, rel_err(g["v"], o.v)
    assert np.abs(g["x"] - o.x).max() < 1e-13 * np.abs(o.x).max()


def test_dense_mean_pressure_200_steps_at_1m(all_cores, dense1m):
    """The mixed form's accuracy gate where contacts exist: mean pressure within 1e-6 (relative) of the
    FP64 oracle after 200 steps of the contact-dense 1M-sphere servo run; the FP64 form within 1e-10."""
    import taichimps_gb300 as G
    steps = 200
    res = {}
    for prec in ("mixed", "fp64"):
        sim, osim = _dense_pair(G, all_cores, dense1m, prec)
        sim.run(steps)
        res[prec] = np.array(sim.fixes[-1].last_pressure(), dtype=np.float64)
        del sim
    osim.run(steps)
    po = np.array(osim.last_pressure, dtype=np.float64)
    mean = lambda t: (t[0] + t[1] + t[2]) / 3.0
    assert mean(po) > 0.5
    err = {k: abs(mean(v) - mean(po)) / abs(mean(po)) for k, v in res.items()}
    print("mean pressure relative error after 200 steps, dense 1M:", {k: f"{v:.2e}" for k, v in err.items()})
    assert err["fp64"] < 1e-10, err
    assert err["mixed"] < 1e-6, err
