"""The product kernels' launch-shape autotuner, host side (no GPU).

hbi_construct_lh times every compiled launch shape of the phase kernels on
the operator (five launches per phase after a warm-up) and keeps, per phase,
the shape with the lowest median time; a later shape must beat the earlier
best by more than 1% (near-ties keep the default, shape 0).  These tests run
that selection rule on recorded timings and check the shape table against
the kernels' shared-memory and chunk-width limits.
"""
import numpy as np
import pytest

import hbi_gb300 as H

# the median phase times (us) that construct_LH recorded for every shape on
# a GB300 (c2 shear operator, 65,536 elements, FP32 store; five launches per
# shape): phase 1 in the order of stream_shapes(1) -- 12, 8 and 6 warps with
# the row mapping, then the same with one lane per column -- and phase 2 in
# the order of stream_shapes(2)
RECORDED = {
    "phase1": [88.0, 102.3, 114.62, 71.62, 79.78, 83.94],
    "phase2": [67.46, 77.7, 81.79, 69.54, 77.7],
}


def test_selection_on_recorded_timings():
    b1, m1 = H.autotune_select([[t] for t in RECORDED["phase1"]])
    b2, m2 = H.autotune_select([[t] for t in RECORDED["phase2"]])
    assert b1 == 3 and b2 == 0
    assert m1[3] == pytest.approx(71.62) and m2[0] == pytest.approx(67.46)


def test_median_ignores_one_outlier_and_invalid_runs():
    t = [[50.0, 50.2, 49.9, 50.1, 50.0], [45.0, 45.1, 900.0, 44.9, 45.2]]
    assert H.autotune_select(t)[0] == 1
    t = [[50.0, -1.0, float("nan"), 50.1, 50.0], [float("inf"), 0.0, -1.0, float("nan"), -2.0]]
    best, med = H.autotune_select(t)
    assert best == 0 and med[1] == -1.0
    with pytest.raises(H.HBIError):
        H.autotune_select([[-1.0, 0.0], [float("nan"), -5.0]])


def test_near_ties_keep_the_earlier_shape():
    assert H.autotune_select([[100.0] * 5, [99.5] * 5, [99.2] * 5])[0] == 0
    assert H.autotune_select([[100.0] * 5, [98.0] * 5, [97.5] * 5])[0] == 1
    assert H.autotune_select([[100.0] * 5, [98.0] * 5, [96.9] * 5])[0] == 2


def test_shape_table_fits_the_kernels():
    for phase in (1, 2):
        shapes = H.stream_shapes(phase)
        assert len(shapes) >= 3 and shapes[0] == (12, 2, 8192, 0, 0)
        for nw, ns, sb, variant, sched in shapes:
            assert 1 <= nw <= 32 and ns >= 2 and sb in (8192, 16384)
            assert variant in (0, 1) and sched in (0, 1, 2, 3)
            smem = nw * ns * sb + nw * 128 * 8 + nw * ns * 8
            assert smem <= 227 * 1024
            for esz in (2, 4, 8):
                for ntp in range(16 // esz, 512 // esz + 1, 16 // esz):
                    cc = (sb // (ntp * esz)) // 16 * 16
                    cc = min(cc, 128)
                    assert 16 <= cc <= 128 and cc * ntp * esz <= sb
    assert {m for _, _, _, m, _ in H.stream_shapes(1)} == {0, 1}
    # every schedule is a candidate of both phases
    for phase in (1, 2):
        assert {s for *_, s in H.stream_shapes(phase)} == {0, 1, 2, 3}


@pytest.mark.parametrize("nblocks,nw", [(1, 12), (7, 3), (152, 12)])
def test_block_schedule_is_local_and_balanced(nblocks, nw):
    """The schedule with locality: every item exactly once; each block's items
    are consecutive in store order; block loads within one item of the
    average; inside a block every warp's items in decreasing cost."""
    rng = np.random.default_rng(nblocks + nw)
    n = 5000
    cost = rng.integers(512, 300_000, n)
    key = rng.permutation(n).astype(np.int64) * 4096
    woff, witem = H.plan_block_schedule(cost, key, nblocks, nw)
    assert woff[0] == 0 and woff[-1] == n and np.all(np.diff(woff) >= 0)
    assert np.array_equal(np.sort(witem), np.arange(n))
    rank = np.empty(n, dtype=np.int64)
    rank[np.argsort(key, kind="stable")] = np.arange(n)
    loads = []
    for b in range(nblocks):
        items = witem[woff[b * nw]:woff[(b + 1) * nw]]
        if len(items):
            r = np.sort(rank[items])
            assert r[-1] - r[0] + 1 == len(r)  # a run of consecutive items
        loads.append(cost[items].sum())
        for w in range(nw):
            c = cost[witem[woff[b * nw + w]:woff[b * nw + w + 1]]]
            assert np.all(np.diff(c) <= 0)
    loads = np.array(loads)
    assert np.abs(loads - cost.sum() / nblocks).max() <= cost.max()


def _vswz(c, nv):
    g = min(nv & -nv, 8)
    shift = {8: 0, 4: 1, 2: 2, 1: 3}[g]
    return (c >> shift) & (g - 1)


@pytest.mark.parametrize("nv", list(range(1, 33)))
def test_v_store_swizzle_is_conflict_free_and_in_bounds(nv):
    """The V-store swizzle (vswz in hbi_structure.hpp): within a column segment
    of nv 16-byte vectors it permutes the vectors, and eight consecutive
    columns reading the same logical vector hit eight different 16-byte bank
    slots of shared memory (vector address mod 8)."""
    for c in range(64):
        s = _vswz(c, nv)
        assert sorted(k ^ s for k in range(nv)) == list(range(nv))
    for c0 in range(0, 64, 8):
        for k in range(nv):
            slots = {((c0 + c) * nv + (k ^ _vswz(c0 + c, nv))) % 8 for c in range(8)}
            assert len(slots) == 8, (nv, c0, k)
