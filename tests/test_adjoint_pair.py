"""
The differentiable run's per-contact forward and hand-written reverse
(taichimps_gb300/csrc/tmps_adjoint.cuh), compiled for the host by g++, against
PyTorch autograd of the same contact law (tests/_adjoint_torch.py): stick,
slip, slip with zero shear, the limit_damping clamp, rows out of contact, with
and without the history update.  No GPU.
"""

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

from _adjoint_torch import torch_pair

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("adj") / "libpair_harness.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    str(HERE / "adjoint" / "pair_harness.cpp"), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    dp = ctypes.POINTER(ctypes.c_double)
    lib.harness_pair_forward.argtypes = [dp, ctypes.c_int, dp, dp]
    lib.harness_pair_reverse.argtypes = [dp, ctypes.c_int, dp, dp, dp]
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _cases(rng, n, shear_scale, sep_scale=0.0, zero_shear=False):
    """Rows of (d, ra, rb, ma, mb, va, vb, wa, wb, sh) = 22 numbers each."""
    rows = []
    for _ in range(n):
        ra, rb = rng.uniform(0.4, 0.6, 2)
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        overlap = rng.uniform(-0.02, 0.06)  # some rows out of contact
        d = u * (ra + rb) * (1.0 - overlap)
        ma, mb = 2.5 * 4.0 / 3.0 * np.pi * np.array([ra, rb]) ** 3
        va, vb = rng.normal(size=3), rng.normal(size=3)
        va += sep_scale * u
        wa, wb = rng.normal(size=3), rng.normal(size=3)
        sh = np.zeros(3) if zero_shear else rng.normal(size=3) * shear_scale
        rows.append(np.concatenate([d, [ra, rb, ma, mb], va, vb, wa, wb, sh]))
    return np.array(rows)


PARAMS = dict(kn=1.0e5, kt=1.0e5 * 2.0 / 7.0, gamman=50.0, gammat=25.0, xmu=0.5, dt=5e-5)


def _torch_vjp(rows, bars, shearupdate, limit_damping):
    n = len(rows)
    T = lambda a: torch.tensor(a, dtype=torch.float64, requires_grad=True)
    d, ra, rb, ma, mb = T(rows[:, 0:3]), T(rows[:, 3]), T(rows[:, 4]), T(rows[:, 5]), T(rows[:, 6])
    va, vb, wa, wb, sh = T(rows[:, 7:10]), T(rows[:, 10:13]), T(rows[:, 13:16]), T(rows[:, 16:19]), T(rows[:, 19:22])
    kn, gamman, gammat, xmu = (T(np.full(n, PARAMS[k])) for k in ("kn", "gamman", "gammat", "xmu"))
    kt = T(np.full((n, 1), PARAMS["kt"]))
    P = dict(kn=kn, kt=kt, gamman=gamman, gammat=gammat, xmu=xmu, dt=PARAMS["dt"], limit_damping=limit_damping)
    F, tor, sh_out, mask = torch_pair(P, shearupdate, d, ra, rb, ma, mb, va, vb, wa, wb, sh)
    b = torch.tensor(bars, dtype=torch.float64)
    fa, fb, ta, tb, w, shb = b[:, 0:3], b[:, 3:6], b[:, 6:9], b[:, 9:12], b[:, 12:18], b[:, 18:21]
    vir = torch.stack([d[:, 0] * F[:, 0], d[:, 1] * F[:, 1], d[:, 2] * F[:, 2],
                       d[:, 0] * F[:, 1], d[:, 0] * F[:, 2], d[:, 1] * F[:, 2]], dim=1)
    L = ((fa * F).sum() - (fb * F).sum() + (ta * (-ra[:, None] * tor)).sum() + (tb * (-rb[:, None] * tor)).sum()
         + (w * vir).sum() + (shb * sh_out).sum())
    L.backward()
    g = np.zeros((n, 24))
    g[:, 0:3] = d.grad.numpy()
    g[:, 3:6] = va.grad.numpy()
    assert np.allclose(va.grad.numpy(), -vb.grad.numpy(), rtol=0, atol=1e-12 * (1 + np.abs(va.grad.numpy()).max()))
    g[:, 6:9], g[:, 9:12] = wa.grad.numpy(), wb.grad.numpy()
    g[:, 12], g[:, 13], g[:, 14], g[:, 15] = ra.grad.numpy(), rb.grad.numpy(), ma.grad.numpy(), mb.grad.numpy()
    g[:, 16:19] = sh.grad.numpy()
    g[:, 19], g[:, 20], g[:, 21] = kn.grad.numpy(), kt.grad.numpy()[:, 0], gamman.grad.numpy()
    g[:, 22], g[:, 23] = gammat.grad.numpy(), xmu.grad.numpy()
    out = torch.cat([F, tor, sh_out], dim=1).detach().numpy()
    return out, g, mask.numpy()


@pytest.mark.parametrize("shearupdate", [1, 0])
@pytest.mark.parametrize("kind", ["mixed", "zero_shear", "clamp"])
def test_pair_reverse_matches_autograd(harness, shearupdate, kind):
    rng = np.random.default_rng([7, shearupdate, len(kind)])
    limit = 0
    if kind == "mixed":
        rows = np.concatenate([_cases(rng, 40, 1e-3), _cases(rng, 40, 3e-2)])
    elif kind == "zero_shear":
        rows = _cases(rng, 60, 0.0, zero_shear=True)
    else:
        rows = _cases(rng, 60, 1e-2, sep_scale=200.0)
        limit = 1
    bars = rng.normal(size=(len(rows), 21))
    p = np.array([PARAMS["kn"], PARAMS["kt"], PARAMS["gamman"], PARAMS["gammat"], PARAMS["xmu"], PARAMS["dt"],
                  float(limit)])
    out_t, g_t, mask_t = _torch_vjp(rows, bars, bool(shearupdate), limit)
    masks = []
    for k, row in enumerate(rows):
        a = np.ascontiguousarray(row)
        out = np.zeros(9)
        m = harness.harness_pair_forward(_ptr(p), shearupdate, _ptr(a), _ptr(out))
        masks.append(m)
        assert m == mask_t[k], (k, m, mask_t[k])
        np.testing.assert_allclose(out, out_t[k], rtol=1e-12, atol=1e-12 * (1 + np.abs(out_t[k]).max()))
        g = np.zeros(24)
        b = np.ascontiguousarray(bars[k])
        harness.harness_pair_reverse(_ptr(p), shearupdate, _ptr(a), _ptr(b), _ptr(g))
        scale = 1.0 + np.abs(g_t[k]).max()
        np.testing.assert_allclose(g, g_t[k], rtol=1e-10, atol=1e-10 * scale, err_msg=f"row {k} mask {m}")
    masks = np.array(masks)
    # the cases reach the branches they are meant to
    assert (masks & 1).sum() > 0 and ((masks & 1) == 0).sum() > 0
    if kind == "mixed":
        assert ((masks & 3) == 3).sum() > 0 and ((masks & 3) == 1).sum() > 0
    if kind == "zero_shear" and shearupdate == 0:
        assert ((masks & 7) == 3).sum() > 0          # slip with |shear| = 0: no tangential force
    if kind == "clamp":
        assert (masks & 8).sum() > 0
