"""
The neighbor build decides most candidate pairs with an FP32 test on
cell-local offsets and sends only those within a slack of the cut to the
reference's exact FP64 test (tmps_nlist.cu, k_build; neighbor.py:329-351).
The slack is meant to exceed the FP32 error by a wide margin, so a pair the
FP32 test drops is out of reach for the FP64 test too, and a pair it takes
without the FP64 test is within reach for it.

This restates k_build's FP32 arithmetic in numpy float32 (with and without
fused multiply-adds, either of which the compiler may emit) on pairs placed
at the cut to within a few parts in 1e5, across periodic boundaries and
boxes far from the origin, and checks both implications against the FP64
test.  CPU only.
"""

import numpy as np

f32 = np.float32


def _fma(a, b, c):
    # one rounding of the exact a*b + c (a float32 product is exact in float64)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def _fp32_decisions(oi, oj, off, h32, hsum, ri32, rj32, skin32, fused):
    d = [((oi[:, k] - oj[:, k]) - off[:, k].astype(f32) * h32[k]).astype(f32) for k in range(3)]
    if fused:
        rq = _fma(d[2], d[2], _fma(d[1], d[1], (d[0] * d[0]).astype(f32)))
    else:
        rq = ((d[0] * d[0] + d[1] * d[1]).astype(f32) + (d[2] * d[2]).astype(f32)).astype(f32)
    mi = np.max(np.abs(oi), axis=1).astype(f32)
    mj = np.max(np.abs(oj), axis=1).astype(f32)
    cut = ((ri32 + rj32).astype(f32) + skin32).astype(f32)
    slack = (f32(1e-5) * (((hsum + mi) + mj) + cut)).astype(f32)
    lim = (cut + slack).astype(f32)
    near = (cut - slack).astype(f32)
    out = ~(rq < (lim * lim).astype(f32))
    inside = (near > 0) & (rq < (near * near).astype(f32))
    return out, inside


def test_fp32_decisions_agree_with_the_fp64_test():
    rng = np.random.default_rng(2026)
    skin = 0.1
    checked_band = 0
    for trial in range(12):
        prd = rng.uniform(6.0, 220.0, size=3)
        lo = rng.uniform(-150.0, 150.0, size=3)
        per = rng.integers(0, 2, size=3)
        m = 200_000
        ri = rng.uniform(0.3, 0.6, size=m)
        rj = rng.uniform(0.3, 0.6, size=m)
        rad = (ri + rj) + skin
        csize = 1.3  # at least the largest cut
        g = np.maximum(np.floor(prd / csize).astype(np.int64), 3)
        h = prd / g
        xi = lo + rng.uniform(0.0, 1.0, size=(m, 3)) * prd
        u = rng.normal(size=(m, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        # at the cut to within a few parts in 1e5, some further out and in
        eps = np.where(rng.uniform(size=m) < 0.8, rng.uniform(-4e-5, 4e-5, size=m), rng.uniform(-0.3, 0.05, size=m))
        xj = xi + u * (rad * (1.0 + eps))[:, None]
        keep = np.ones(m, dtype=bool)
        for k in range(3):
            if per[k]:
                xj[:, k] = lo[k] + np.mod(xj[:, k] - lo[k], prd[k])
            else:
                keep &= (xj[:, k] >= lo[k]) & (xj[:, k] < lo[k] + prd[k])

        def cell(x):
            lam = (x - lo) / prd
            return np.clip(np.floor(lam * g).astype(np.int64), 0, g - 1)

        ci, cj = cell(xi), cell(xj)
        off = cj - ci
        for k in range(3):
            if per[k]:
                off[:, k] = np.where(off[:, k] == g[k] - 1, -1, off[:, k])
                off[:, k] = np.where(off[:, k] == -(g[k] - 1), 1, off[:, k])
        keep &= np.all(np.abs(off) <= 1, axis=1)
        xi, xj, ri, rj, off, ci, cj = xi[keep], xj[keep], ri[keep], rj[keep], off[keep], ci[keep], cj[keep]
        # cell-local FP32 offsets as k_permute forms them
        oi = (xi - (lo + ci * h)).astype(f32)
        oj = (xj - (lo + cj * h)).astype(f32)
        h32 = (prd / g).astype(f32)
        hsum = f32(h32[0] + h32[1]) + h32[2]
        # the exact FP64 test (minimum image, neighbor.py:329-351)
        d = xi - xj
        for k in range(3):
            if per[k]:
                d[:, k] -= prd[k] * np.round(d[:, k] / prd[k])
        rsq = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        ref_in = rsq < ((ri + rj) + skin) ** 2
        for fused in (False, True):
            out, inside = _fp32_decisions(oi, oj, off, h32, hsum, ri.astype(f32), rj.astype(f32), f32(skin), fused)
            assert not np.any(out & ref_in), "FP32 test dropped a pair within the cut"
            assert not np.any(inside & ~ref_in), "FP32 test took a pair beyond the cut"
            checked_band += int(np.count_nonzero(~out & ~inside))
        # both sides of the cut are well represented
        assert ref_in.sum() > 0.3 * len(ref_in) and (~ref_in).sum() > 0.3 * len(ref_in)
    # and some pairs are close enough to the cut to need the FP64 test
    assert checked_band > 1000


def approx_f32(x):
    """The device's approx_f32 (tmps_common.cuh): sign, rebiased exponent and the top 20 significand
    bits of a double, truncated, as an FP32 value; zero below the FP32 normal range."""
    hi = (np.asarray(x, dtype=np.float64).view(np.uint64) >> np.uint64(32)).astype(np.int64)
    sign = hi & 0x80000000
    e = (hi >> 20) & 0x7FF
    m = hi & 0xFFFFF
    ef = e - 1023 + 127
    bits = np.where(e == 0x7FF, sign | 0x7F800000 | np.where(m != 0, 0x400000, 0),
                    np.where(ef <= 0, sign, np.where(ef >= 255, sign | 0x7F800000, sign | (ef << 23) | (m << 3))))
    return bits.astype(np.uint32).view(f32)


def test_approx_f32_truncates_within_2e_20():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-1e4, 1e4, 100_000), rng.normal(size=100_000) * 1e-3,
                        [0.0, -0.0, 1.0, -1.0, 1e-300, 1e300, np.inf, -np.inf]])
    a = approx_f32(x)
    fin = np.isfinite(x) & (np.abs(x) > 1e-37) & (np.abs(x) < 1e38)
    rel = np.abs(a[fin].astype(np.float64) - x[fin]) / np.abs(x[fin])
    assert rel.max() < 2.0 ** -20
    assert np.all(np.abs(a[fin]) <= np.abs(x[fin]))  # truncation toward zero
    assert a[-8] == 0.0 and a[-6] == 1.0 and a[-5] == -1.0 and a[-4] == 0.0
    assert a[-3] == f32(np.inf) and a[-2] == f32(np.inf) and a[-1] == -f32(np.inf)
    assert np.isnan(approx_f32(np.array([np.nan])))[0]


def test_fp32_gap_bound_is_a_lower_bound():
    """The contact bound (tmps_fused.cu, k_bounds) takes the FP64 difference of the positions to FP32 by
    truncation (approx_f32), forms the periodic image, distance and gap in FP32 and lowers the gap by
    3e-6 of the magnitudes involved (the separation before the image, the image shift, r and the radii):
    it must never exceed the FP64 gap, or a group could be ruled out while one of its pairs can still
    close.  Pairs at the contact distance within 1e-3, atoms up to 1e4 from the origin, partners seen
    through periodic images of a box of ~1.2e3 (a listed pair is never near half a box)."""
    rng = np.random.default_rng(7)
    m = 400_000
    prd = np.array([1200.0, 1100.0, 1300.0])
    r = np.concatenate([rng.uniform(0.0, 1.5, size=m // 2), rng.uniform(0.5, 0.7, size=m // 2)])
    u = rng.normal(size=(m, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    d = u * r[:, None] * rng.uniform(0.999, 1.001, size=(m, 1))
    ri = rng.uniform(0.25, 0.6, size=m)
    rj = rng.uniform(0.25, 0.6, size=m)
    scale = np.where(rng.uniform(size=m) < 0.5, 1e4, 50.0)
    xi = rng.uniform(-1.0, 1.0, size=(m, 3)) * scale[:, None]
    img = np.where(rng.uniform(size=(m, 3)) < 0.5, 0, rng.integers(-2, 3, size=(m, 3)))
    xj = (xi - d) + img * prd          # the partner, in half the cases seen through a periodic image
    dd = xi - xj                       # the FP64 difference the kernel forms
    ex = dd - np.rint(dd / prd) * prd  # the exact minimum image
    exact = np.sqrt((ex ** 2).sum(axis=1)) - (ri + rj)
    prd32, iprd32 = approx_f32(prd), approx_f32(1.0 / prd)
    for fused in (False, True):
        fd, mag = [], np.zeros(m, dtype=f32)
        for c in range(3):
            x = approx_f32(dd[:, c])
            mag = (mag + np.abs(x)).astype(f32)
            nimg = np.rint((x * iprd32[c]).astype(f32)).astype(f32)
            x = _fma(-nimg, np.full_like(x, prd32[c]), x) if fused else (x - (nimg * prd32[c]).astype(f32)).astype(f32)
            mag = (mag + (np.abs(nimg) * prd32[c]).astype(f32)).astype(f32)
            fd.append(x)
        if fused:
            rq = _fma(fd[2], fd[2], _fma(fd[1], fd[1], (fd[0] * fd[0]).astype(f32)))
        else:
            rq = ((fd[0] * fd[0] + fd[1] * fd[1]).astype(f32) + (fd[2] * fd[2]).astype(f32)).astype(f32)
        rf = np.sqrt(rq.astype(f32)).astype(f32)
        rs = (approx_f32(ri) + approx_f32(rj)).astype(f32)
        tot = ((mag + rf).astype(f32) + rs).astype(f32)
        gp = ((rf - rs).astype(f32) - (f32(3e-6) * tot).astype(f32)).astype(f32)
        assert np.all(gp.astype(np.float64) <= exact), "FP32 gap above the FP64 gap"
        # and not needlessly low: within 6e-6 of the magnitudes
        assert np.all(exact - gp <= 6e-6 * tot + 1e-12)
        # interior pairs keep a tight bound
        inner = np.all(img == 0, axis=1)
        assert np.all(exact[inner] - gp[inner] <= 2e-5)
