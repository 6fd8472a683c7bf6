"""
CPU-only checks of the boundary and the host logic (no GPU calls):
the C-ABI library loads and exports every entry point include/taichimps_gb300.h
declares; the ctypes struct layouts match the C header byte for byte; the
host-side grid setup agrees with the oracle's restatement; validation errors.
"""

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "taichimps_gb300.h"


def header_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tmps_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from taichimps_gb300 import _lib
    L = _lib.load()
    declared = header_functions()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(L, name), f"{name} declared in the header but not exported"
    assert set(declared) == set(_lib.exported_symbols()), "ctypes signatures out of step with the header"
    assert L.tmps_version().decode().startswith("taichimps_gb300")


def test_struct_layouts_match_header(tmp_path):
    from taichimps_gb300 import _lib
    structs = {"tmps_box": _lib.Box, "tmps_atoms": _lib.Atoms, "tmps_nlist": _lib.NList,
               "tmps_pair_params": _lib.PairParams, "tmps_servo": _lib.Servo, "tmps_engine": _lib.Engine,
               "tmps_instance": _lib.Instance, "tmps_adj_params": _lib.AdjParams, "tmps_adj_servo": _lib.AdjServo,
               "tmps_adj_rec": _lib.AdjRec, "tmps_adj_sys": _lib.AdjSys, "tmps_adj_tape": _lib.AdjTape,
               "tmps_adj_bar": _lib.AdjBar, "tmps_wall_params": _lib.WallParams}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.split() for line in out if line.strip())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


@pytest.mark.parametrize("prd,per,rmax,skin", [
    ((17.42, 17.42, 17.42), (1, 1, 1), 0.55, 0.1),
    ((106.56, 106.56, 106.56), (1, 1, 1), 0.6, 0.1),
    ((20.0, 20.0, 20.0), (0, 0, 0), 1.0, 0.2),
    ((2.5, 3.3, 4.0), (1, 1, 1), 0.5, 0.1),
    ((0.0075, 0.0075, 0.0075), (1, 1, 1), 5e-4, 2e-4),
    ((1000.0, 3.0, 3.0), (1, 0, 1), 0.5, 0.05),
])
def test_grid_setup_matches_oracle(oracle, prd, per, rmax, skin):
    from taichimps_gb300.neighbor import setup_grid_dims
    g, cs = setup_grid_dims(prd, per, 2.0 * rmax, skin, 200000)
    dom = oracle.OracleDomain.make([0.0] * 3, list(prd), tuple("p" if p else "f" for p in per))
    og = np.zeros(3, dtype=np.int32)
    ocs = np.zeros(3)
    oracle.lib().or_setup_grid(ctypes.byref(dom.cbox()), ctypes.c_double(2.0 * rmax), ctypes.c_double(skin),
                               200000, oracle._p(og, oracle._i32p), oracle._p(ocs))
    np.testing.assert_array_equal(g, og)
    np.testing.assert_array_equal(cs, ocs)


def test_morton_rank_is_permutation():
    from taichimps_gb300.neighbor import morton_rank
    for dims in ((1, 1, 1), (3, 5, 7), (16, 16, 16), (58, 58, 58)):
        r = morton_rank(*dims)
        assert sorted(r.tolist()) == list(range(int(np.prod(dims))))
    r = morton_rank(2, 2, 2)
    assert r[0] == 0 and r[1] == 1 and r[2] == 2 and r[4] == 4  # x fastest, then y, then z


def test_granular_derivations_cpu():
    """tests/test_pair_granular_parsing.py:56-85 for the package's PairGranular (host logic only)."""
    import math
    from taichimps_gb300.GRANULAR.granular import PairGranular, mix_stiffness_e, mix_stiffness_g
    E, P, COR, FRIC = 71.6e9, 0.23, 0.95, 0.3
    pair = PairGranular(None, normal="hertz/material", normal_coeffs=[E, COR, P], tangential="mindlin",
                        tangential_coeffs=[None, 1.0, FRIC], damping="coeff_restitution")
    np.testing.assert_allclose(pair.kn, 4.0 / 3.0 * mix_stiffness_e(E, E, P, P), rtol=1e-12)
    np.testing.assert_allclose(pair.kt, 8.0 * mix_stiffness_g(E, E, P, P), rtol=1e-12)
    logcor = math.log(COR)
    np.testing.assert_allclose(pair.damp, -1.22474487139158894067 * 1.82574185835055380345 * logcor
                               / math.sqrt(math.pi ** 2 + logcor ** 2), rtol=1e-12)
    assert pair.params.style == 4 and pair.params.tangential_id == 3
    with pytest.raises(ValueError, match="jkr"):
        PairGranular(None, normal="jkr", normal_coeffs=[1e9, 0.95, 0.23, 0.1])
    with pytest.raises(ValueError, match="restitution"):
        PairGranular(None, normal="hertz", normal_coeffs=[1e5, 1.5], damping="tsuji")


def test_deform_validation_cpu():
    from taichimps_gb300.EXTRA_FIX.deform_pressure import FixDeformPressure
    with pytest.raises(ValueError, match="gain"):
        FixDeformPressure(None, axes={"x": {"style": "pressure", "ptarget": 1.0, "pgain": 0.0}})
    with pytest.raises(ValueError, match="couple"):
        FixDeformPressure(None, axes={"x": {"style": "erate", "rate": 0.1}}, couple="xy")
    # the reference's validation of the volume and box styles (deform_pressure.py:316-385)
    with pytest.raises(ValueError, match="at least one other deformed dimension"):
        FixDeformPressure(None, axes={"x": {"style": "volume"}})
    with pytest.raises(ValueError, match="vol/balance/p only applies"):
        FixDeformPressure(None, axes={"x": {"style": "erate", "rate": 0.1}}, vol_balance_p=True)
    with pytest.raises(ValueError, match="two dimensions holding the volume"):
        FixDeformPressure(None, axes={"x": {"style": "volume"}, "z": {"style": "erate", "rate": 0.1}},
                          vol_balance_p=True)
    with pytest.raises(ValueError, match="box may only be combined"):
        FixDeformPressure(None, axes={"x": {"style": "final", "flo": 0.0, "fhi": 1.0}}, box={"style": "volume"})
    with pytest.raises(ValueError, match="constant volume and a mean"):
        FixDeformPressure(None, axes={"x": {"style": "volume"}, "z": {"style": "pressure/mean", "ptarget": 1.0,
                                                                      "pgain": 1e-3}})
    with pytest.raises(NotImplementedError):
        FixDeformPressure(None, axes={"x": {"style": "variable"}})
    with pytest.raises(NotImplementedError):
        FixDeformPressure(None, axes={"xy": {"style": "erate", "rate": 0.1}})
    with pytest.raises(ValueError, match="nvt/sllod"):
        FixDeformPressure(None, axes={"x": {"style": "erate/rescale"}})


def test_product_path_fails_loudly_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import taichimps_gb300 as G
    with pytest.raises(RuntimeError, match="CUDA device"):
        G.AtomSystem(max_atoms=4)
