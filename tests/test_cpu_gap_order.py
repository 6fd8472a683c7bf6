"""
The ordered pass of the contact kernel (tmps_fused.cu, cf_body): after the
first pass that follows the contact bounds, C walks the 32-atom groups in
ascending order of their gap bound (k_gap_keys / k_bitonic_* / k_gap_order),
warp w taking positions w + 32 W b + lane W (W warps, b = 0, 1, ...) and
stopping at its first base with no live lane.  Because the threshold only
grows between builds, the live groups are a prefix of that order, and the
walk must visit exactly the groups whose gap does not exceed the threshold.

This restates the key transform and the walk in numpy and checks the visited
set against the definition of a live group, for gap arrays with ties,
infinities and NaNs, group counts around the warp and base boundaries, and
several thresholds.  CPU only.
"""

import numpy as np
import pytest


def _keys(gap: np.ndarray) -> np.ndarray:
    """k_gap_keys: the gap's bits made to order as unsigned (a NaN first), then the group."""
    u = gap.astype(np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    neg = (u & 0x80000000) != 0
    k = np.where(neg, (~u) & 0xFFFFFFFF, u | 0x80000000)
    k = np.where(nan, 0, k)
    return (k << np.uint64(32)) | np.arange(len(gap), dtype=np.uint64)


def _walk(order: np.ndarray, sgap: np.ndarray, thr: np.float32, nwarps: int) -> set:
    ng = len(order)
    visited = set()
    for gw in range(nwarps):
        base = gw
        while base < ng:
            k = base + np.arange(32) * nwarps
            ok = k < ng
            live = np.zeros(32, dtype=bool)
            live[ok] = ~(sgap[k[ok]] > thr)
            if not live.any():
                break
            visited.update(int(g) for g in order[k[live]])
            base += 32 * nwarps
    return visited


@pytest.mark.parametrize("ng,nwarps", [(1, 1), (31, 4), (32, 1), (33, 8), (1000, 64), (4097, 1824), (31250, 1824)])
def test_ordered_walk_visits_exactly_the_live_groups(ng, nwarps):
    rng = np.random.default_rng(ng * 7 + nwarps)
    gap = rng.uniform(-0.05, 0.15, size=ng).astype(np.float32)
    # ties, groups without neighbors, pinned groups, NaN bounds
    gap[rng.integers(0, ng, size=max(1, ng // 10))] = np.float32(0.01)
    gap[rng.integers(0, ng, size=max(1, ng // 20))] = np.float32(3e38)
    gap[rng.integers(0, ng, size=max(1, ng // 20))] = np.float32(-3e38)
    if ng > 3:
        gap[rng.integers(0, ng, size=2)] = np.float32(np.nan)
    keys = np.sort(_keys(gap))  # distinct keys: any correct sort gives this order
    order = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    sgap = gap[order]
    assert sorted(order.tolist()) == list(range(ng))
    for thr in (np.float32(-1.0), np.float32(0.0), np.float32(0.01), np.float32(0.05), np.float32(np.inf),
                np.float32(np.nan)):
        live = {g for g in range(ng) if not (gap[g] > thr)}
        assert _walk(order, sgap, thr, nwarps) == live, (ng, nwarps, thr)


def test_live_groups_are_a_prefix_of_the_order():
    rng = np.random.default_rng(3)
    gap = rng.normal(0.02, 0.05, size=5000).astype(np.float32)
    gap[::97] = np.float32(np.nan)
    order = (np.sort(_keys(gap)) & np.uint64(0xFFFFFFFF)).astype(np.int64)
    for thr in np.linspace(-0.2, 0.3, 41).astype(np.float32):
        live = ~(gap[order] > thr)
        first_out = np.argmin(live) if not live.all() else len(live)
        assert live[:first_out].all() and not live[first_out:].any()
