"""The streamed product's work plan (row-tiled stores, bulk-copy items,
partials, phase-3 gather) walked on the host by hbi_plan_emulate, against the
oracle's product on the same HACApK-packed factors.  No GPU: this checks the
plan's bounds and index arithmetic before any kernel reads it.

Tolerance: 1e-12 relative (the plan sums in a different order than the
oracle's leaf loop)."""
import numpy as np
import pytest

import hbi_gb300 as H
from hbi_gb300 import mesh
from gpu_cases import case, oracle_geometry


def _random_factors(oracle, coord, seed, kmax=24):
    lod, leaves, _ = oracle.build_structure(coord)
    rng = np.random.default_rng(seed)
    lv = np.array(leaves, dtype=np.int32)
    n = len(coord)
    lr = lv[:, 0] == 1
    lv[lr, 1] = rng.integers(0, kmax + 1, lr.sum())  # ranks, some zero
    sizes = np.where(lv[:, 0] == 1, lv[:, 1] * (lv[:, 3] + lv[:, 5]), lv[:, 3] * lv[:, 5]).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(sizes)])
    body = rng.standard_normal(int(off[-1]))
    return n, lv, off, body


@pytest.mark.parametrize("vec", [2, 4, 8])
@pytest.mark.parametrize("shape", [(64, 32), (150, 30), (40, 40)])
def test_plan_matches_oracle_product(oracle, vec, shape):
    xcol, ycol, zcol, _, _ = mesh.mesh_3ddip(shape[0], shape[1], 0.1, 30.0)
    coord = np.stack([xcol, ycol, zcol], 1)
    n, lv, off, body = _random_factors(oracle, coord, seed=shape[0] + vec)
    Ho = oracle.HMatrix.from_body(n, lv, off, body)
    x = np.random.default_rng(1).standard_normal(n)
    y_ref = Ho.matvec(x)
    y, st = H.plan_emulate(n, lv, body, vec, x)
    assert np.linalg.norm(y - y_ref) <= 1e-12 * np.linalg.norm(y_ref)
    assert st["items1"] > 0 and st["items2"] > 0


def test_plan_2dvs_and_small(oracle):
    for n in (17, 100, 1024):
        xel, xer, xcol, _ = mesh.mesh_2dp(n, 40.0 / n)
        coord = np.stack([xcol, np.zeros(n), np.zeros(n)], 1)
        n, lv, off, body = _random_factors(oracle, coord, seed=n, kmax=8)
        Ho = oracle.HMatrix.from_body(n, lv, off, body)
        x = np.cos(np.arange(n))
        y, _ = H.plan_emulate(n, lv, body, 4, x)
        assert np.allclose(y, Ho.matvec(x), rtol=1e-12, atol=1e-12 * np.abs(Ho.matvec(x)).max())


def test_plan_on_aca_factors(oracle):
    prob, n, g, w, eps = case("3dph")
    coord = np.stack([g["xcol"], g["ycol"], g["zcol"]], 1)
    lod, leaves, _ = oracle.build_structure(coord)
    Ho = oracle.HMatrix(oracle_geometry(oracle, prob, n, g, w, "s"), lod, leaves)
    x = np.random.default_rng(7).standard_normal(n)
    y, _ = H.plan_emulate(n, Ho.leaves, Ho.body, 4, x)
    ref = Ho.matvec(x)
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("shape", [(64, 32), (150, 30), (40, 40), (128, 64)])
def test_tc_plan_matches_oracle_product(oracle, shape):
    """The ensemble's tensor-core plan: canonical BF16 hi+lo stores walked on
    the host.  hi + lo carries ~16 bits of each factor: 1e-4 relative.  The
    128 x 64 plane has column groups taller than the 1,024-row phase-1
    tiles, so their tiles meet in partial sums."""
    xcol, ycol, zcol, _, _ = mesh.mesh_3ddip(shape[0], shape[1], 0.1, 30.0)
    coord = np.stack([xcol, ycol, zcol], 1)
    n, lv, off, body = _random_factors(oracle, coord, seed=shape[1])
    if shape == (128, 64):
        assert max(int(r[5]) for r in lv if r[0] == 1) > 1024
    Ho = oracle.HMatrix.from_body(n, lv, off, body)
    x = np.random.default_rng(2).standard_normal(n)
    ref = Ho.matvec(x)
    y, st = H.tc_plan_emulate(n, lv, body, x)
    assert np.linalg.norm(y - ref) <= 1e-4 * np.linalg.norm(ref)
    assert st["items1"] > 0 and st["items2"] > 0


@pytest.mark.parametrize("nwarps", [1, 7, 1824])
def test_warp_schedule_is_balanced_permutation(nwarps):
    """Longest-processing-time schedule of the product kernels: every item
    exactly once, each warp's items in decreasing cost, and the busiest warp
    within one item of the average (Graham's bound for LPT is 4/3 of the
    optimum; this checks the weaker max <= avg + max item)."""
    rng = np.random.default_rng(nwarps)
    cost = np.concatenate([rng.integers(512, 300_000, 3000), rng.integers(512, 20_000, 7000)])
    woff, witem = H.plan_warp_schedule(cost, nwarps)
    assert woff[0] == 0 and woff[-1] == len(cost) and np.all(np.diff(woff) >= 0)
    assert np.array_equal(np.sort(witem), np.arange(len(cost)))
    loads = np.array([cost[witem[woff[w]:woff[w + 1]]].sum() for w in range(nwarps)])
    assert loads.max() <= cost.sum() / nwarps + cost.max()
    for w in range(nwarps):
        c = cost[witem[woff[w]:woff[w + 1]]]
        assert np.all(np.diff(c) <= 0)
    # deterministic
    w2, i2 = H.plan_warp_schedule(cost, nwarps)
    assert np.array_equal(w2, woff) and np.array_equal(i2, witem)
