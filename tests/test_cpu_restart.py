"""
LAMMPS binary restart files (taichimps_gb300.restart) against files written by
the reference's own writer (tests/golden/make_restart_fixtures.py ran
src/taichimps/restart.py write_restart on the arrays in restart_inputs.npz):

* read_restart recovers every array bit for bit, the pair style and its
  coefficients, and each contact under both atoms (the second copy negated),
  as the reference's round-trip test asserts (tests/test_restart.py:366-442);
* the writer, given the same arrays and contacts in the same order, writes the
  same bytes as the reference's writer;
* our own files round-trip (gran/* pair styles, rolling histories of six
  values per contact, empty systems), and malformed files are refused.
"""

from pathlib import Path

import numpy as np
import pytest

from taichimps_gb300 import restart as R

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def inp():
    return dict(np.load(GOLD / "restart_inputs.npz"))


def _stored(data):
    """{atom index: {partner tag: values}} from the file's NEIGH_HISTORY records."""
    out = {}
    for i, rec in enumerate(data.fix_extra):
        tags, vals = R.parse_neigh_history(rec)
        out[i] = {int(t): vals[k] for k, t in enumerate(tags)}
    return out


def _reference_order_contacts(d):
    """Both-sided contacts in the order the reference's writer appends them: for each atom i
    ascending, its own contacts in order, each followed by the negated copy under its partner."""
    own = [[] for _ in range(len(d["radius"]))]
    for i, j, s in zip(d["c_i"], d["c_j"], d["c_shear"]):
        own[int(i)].append((int(j), s))
    rows, tags, vals = [], [], []
    for i in range(len(own)):
        for j, s in own[i]:
            rows += [i, j]
            tags += [int(d["tag"][j]), int(d["tag"][i])]
            vals += [s, -s]
    return np.array(rows), np.array(tags), np.array(vals)


@pytest.mark.parametrize("name", ["restart_granular.bin", "restart_history_only.bin", "restart_plain.bin"])
def test_reads_reference_files_bit_for_bit(inp, name):
    d = R.read_restart(GOLD / name)
    n = len(inp["radius"])
    assert d.natoms == n and d.timestep == int(inp["timestep"]) and d.dt == float(inp["dt"])
    for k in ("x", "v", "omega", "radius", "rmass", "tag", "atom_type"):
        np.testing.assert_array_equal(getattr(d, k), inp[k])
    assert d.boxlo == list(inp["boxlo"]) and d.boxhi == list(inp["boxhi"])
    assert d.boundary == ("p", "p", "f")
    assert d.ntypes == int(inp["atom_type"].max())
    if name == "restart_granular.bin":
        assert d.pair_style == "granular"
        m = d.pair_settings["models"][0]
        assert m["normal"] == ("hertz/material", [5.0e6, 0.5, 0.3])
        assert m["tangential"] == ("mindlin", [-1.0, 1.0, 0.5])
        assert m["damping"][0] == "coeff_restitution"
    else:
        assert d.pair_style == ""
    if name == "restart_plain.bin":
        assert d.fix_peratom_styles == []
        assert all(len(r) == 0 for r in d.fix_extra)
        return
    assert d.fix_peratom_styles == ["NEIGH_HISTORY"]
    st = _stored(d)
    tags = inp["tag"]
    for i, j, s in zip(inp["c_i"], inp["c_j"], inp["c_shear"]):
        np.testing.assert_array_equal(st[int(i)][int(tags[j])], s)
        np.testing.assert_array_equal(st[int(j)][int(tags[i])], -s)
    assert sum(len(v) for v in st.values()) == 2 * len(inp["c_i"])
    # the bulk form agrees with the per-record parse
    rows, ptag, vals = d.neigh_history()
    assert len(rows) == 2 * len(inp["c_i"])
    for r, t, v in zip(rows, ptag, vals):
        np.testing.assert_array_equal(st[int(r)][int(t)], v)


@pytest.mark.parametrize("name,pair,hist", [("restart_granular.bin", True, True),
                                            ("restart_history_only.bin", False, True),
                                            ("restart_plain.bin", False, False)])
def test_writes_the_reference_writers_bytes(inp, tmp_path, name, pair, hist):
    sub = {"normal": ("hertz/material", [5.0e6, 0.5, 0.3]), "damping": ("coeff_restitution", []),
           "tangential": ("mindlin", [-1.0, 1.0, 0.5]), "rolling": ("none", []), "twisting": ("none", []),
           "heat": ("none", [])}
    out = tmp_path / name
    R.write_restart_arrays(out, x=inp["x"], v=inp["v"], omega=inp["omega"], radius=inp["radius"],
                           rmass=inp["rmass"], tag=inp["tag"], atom_type=inp["atom_type"], boxlo=inp["boxlo"],
                           boxhi=inp["boxhi"], periodicity=inp["periodicity"], timestep=int(inp["timestep"]),
                           dt=float(inp["dt"]),
                           pair_style="granular" if pair else None,
                           pair_settings={"submodels": sub, "limit_damping": 0} if pair else None,
                           contacts=_reference_order_contacts(inp) if hist else None)
    assert out.read_bytes() == (GOLD / name).read_bytes()


def _random_system(rng, n, dnum=3, contacts=True):
    d = dict(x=rng.random((n, 3)) * 5, v=rng.normal(size=(n, 3)), omega=rng.normal(size=(n, 3)),
             radius=rng.uniform(0.4, 0.6, n), rmass=rng.uniform(1, 2, n), tag=np.arange(1, n + 1, dtype=np.int32),
             atom_type=np.ones(n, dtype=np.int32), boxlo=[0.0] * 3, boxhi=[5.0] * 3, periodicity=[1, 1, 1],
             timestep=77, dt=1e-4)
    if contacts and n > 1:
        m = 3 * n
        i = rng.integers(0, n, m)
        j = (i + 1 + rng.integers(0, n - 1, m)) % n
        d["contacts"] = (i, d["tag"][j], rng.normal(size=(m, dnum)))
    return d


@pytest.mark.parametrize("style", ["gran/hooke", "gran/hooke/history", "gran/hertz/history"])
def test_round_trip_legacy_pair_styles(tmp_path, style):
    rng = np.random.default_rng(1)
    d = _random_system(rng, 30)
    s = dict(kn=2e5, kt=2e5 * 2 / 7, gamman=50.0, gammat=25.0, xmu=0.5, dampflag=1, limit_damping=1)
    f = tmp_path / "a.restart"
    R.write_restart_arrays(f, pair_style=style, pair_settings=s, history_style=style, **d)
    r = R.read_restart(f)
    assert r.pair_style == style and r.pair_settings == s
    for k in ("x", "v", "omega", "radius", "rmass", "tag"):
        np.testing.assert_array_equal(getattr(r, k), d[k])
    rows, tags, vals = r.neigh_history()
    i, t, v = d["contacts"]
    order = np.argsort(i, kind="stable")
    np.testing.assert_array_equal(rows, i[order])
    np.testing.assert_array_equal(tags, t[order])
    np.testing.assert_array_equal(vals, v[order])


def test_round_trip_rolling_history(tmp_path):
    """Six values per contact (shear, then rolling displacement): the record length carries dnum."""
    rng = np.random.default_rng(2)
    d = _random_system(rng, 25, dnum=6)
    f = tmp_path / "r.restart"
    R.write_restart_arrays(f, **d)
    r = R.read_restart(f)
    rows, tags, vals = r.neigh_history()
    assert vals.shape[1] == 6
    i, t, v = d["contacts"]
    order = np.argsort(i, kind="stable")
    np.testing.assert_array_equal(vals, v[order])
    k = int(i[order][0])
    tg, vv = R.parse_neigh_history(r.fix_extra[k], dnum=None)
    assert vv.shape[1] == 6
    np.testing.assert_array_equal(vv, v[order][i[order] == k])


def test_round_trip_edge_sizes(tmp_path):
    rng = np.random.default_rng(3)
    for n, contacts in ((0, False), (1, False), (1, True), (2, True)):
        d = _random_system(rng, n, contacts=contacts)
        if contacts and "contacts" not in d:
            d["contacts"] = (np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros((0, 3)))
        f = tmp_path / f"e{n}{contacts}.restart"
        R.write_restart_arrays(f, **d)
        r = R.read_restart(f)
        assert r.natoms == n and len(r.radius) == n and len(r.fix_extra) == n
        np.testing.assert_array_equal(r.x.reshape(-1, 3), np.asarray(d["x"]).reshape(-1, 3))


def test_refuses_malformed_files(tmp_path, inp):
    good = (GOLD / "restart_granular.bin").read_bytes()
    bad = tmp_path / "bad"
    bad.write_bytes(b"not a restart file at all")
    with pytest.raises(ValueError, match="not a LAMMPS restart"):
        R.read_restart(bad)
    bad.write_bytes(good[:len(good) // 2])
    with pytest.raises(ValueError):
        R.read_restart(bad)
    swapped = bytearray(good)
    swapped[16:20] = (0x01000000).to_bytes(4, "little")
    bad.write_bytes(bytes(swapped))
    with pytest.raises(ValueError, match="byte order"):
        R.read_restart(bad)
    with pytest.raises(ValueError, match="not implemented"):
        R.write_restart_arrays(tmp_path / "x", pair_style="lj/cut", pair_settings={}, x=inp["x"], v=inp["v"],
                               omega=inp["omega"], radius=inp["radius"], rmass=inp["rmass"], tag=inp["tag"],
                               atom_type=inp["atom_type"], boxlo=inp["boxlo"], boxhi=inp["boxhi"],
                               periodicity=[1, 1, 1], timestep=0, dt=1e-4)
