"""
The integer-operation double<->float conversions the setup kernels use instead of the FP64 pipe's
(tmps_selftest_arith): bit for bit against the hardware's rounding on random operands over every
exponent, on ties, at the edges of the FP32 range, on zeros, infinities and NaNs.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(which, a):
    import torch
    from taichimps_gb300 import _device, _lib
    L = _device.lib()
    da = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    m = 2 * len(a) if which == 2 else len(a)
    mine = torch.empty(m, dtype=torch.float64, device="cuda")
    hw = torch.empty(m, dtype=torch.float64, device="cuda")
    rc = L.tmps_selftest_arith(which, da.data_ptr(), len(a), mine.data_ptr(), hw.data_ptr(), _device.stream())
    assert rc == _lib.TMPS_OK
    return mine.cpu().numpy(), hw.cpu().numpy()


def _same(mine, hw):
    """Bitwise equal, NaNs of either kind counting as equal."""
    both_nan = np.isnan(mine) & np.isnan(hw)
    eq = (mine.view(np.int64) == hw.view(np.int64)) | both_nan
    return bool(eq.all()), np.flatnonzero(~eq)[:5]


def _operands(rng, n):
    bits = rng.integers(0, 2 ** 63, size=n, dtype=np.int64) * rng.choice([1, -1], size=n)
    wide = bits.view(np.float64)                                   # every exponent, NaNs, infinities
    usual = rng.uniform(-200.0, 200.0, size=n)
    small = rng.uniform(-1.0, 1.0, size=n) * 10.0 ** rng.uniform(-45, -30, size=n)  # around FP32's floor
    big = rng.uniform(-1.0, 1.0, size=n) * 10.0 ** rng.uniform(37, 40, size=n)      # around FP32's top
    f = rng.uniform(-100.0, 100.0, size=n).astype(np.float32).astype(np.float64)
    ulp = np.spacing(f.astype(np.float32)).astype(np.float64)
    ties = f + 0.5 * ulp                                           # exactly between two floats
    near = ties + rng.choice([-1, 1], size=n) * np.spacing(ties)   # just off the tie
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 2.0 ** -149, 2.0 ** -126, 3.4028234663852886e38,
                        3.4028235677973366e38, 1.0, -1.0])
    return np.concatenate([wide, usual, small, big, ties, near, special])


@pytest.mark.parametrize("which", [0, 1, 2])
def test_conversions_match_hardware(gpu, which):
    a = _operands(np.random.default_rng(11 + which), 200_000)
    ok, bad = _same(*_run(which, a))
    assert ok, (which, a[bad // (2 if which == 2 else 1)])
