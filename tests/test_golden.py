"""Committed fixtures (tests/golden/golden_small.npz, made by
tests/golden/make_golden.py from the oracle) against the oracle (CPU) and
against the GPU path through the C ABI.

CPU: the oracle reproduces its fixtures exactly (structure, entries, RK).
GPU: cluster structure bit-exact; 2dvs entries bit-exact, Okada and
triangular entries within 1e-11 of the largest entry; the RK step of the GPU's
own FP64 H-matrix (ACA eps 1e-6) moves the state by the fixture's increment
within 1e-4 relative.
"""
import os

import numpy as np
import pytest

import hbi_gb300 as H
from hbi_gb300 import configs
from gpu_cases import case, oracle_geometry, product_geometry

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_small.npz"))


def test_oracle_reproduces_golden_structure(oracle):
    lod, leaves, _ = oracle.build_structure(G["struct_coord"])
    assert np.array_equal(lod, G["struct_lod"])
    assert np.array_equal(np.array(leaves, dtype=np.int32), G["struct_leaves"])


@pytest.mark.parametrize("kind", ["2dvs", "3dph", "3dnt", "2dph", "2dn", "3dht"])
def test_oracle_reproduces_golden_entries(oracle, kind):
    prob, n, g, w, eps = case(kind, 256 if kind == "2dvs" else None)
    ij = G[f"entry_{kind}_ij"]
    for v in ("s", "n"):
        key = f"entry_{kind}_{v}"
        if key not in G:
            continue
        geo = oracle_geometry(oracle, prob, n, g, w, v)
        got = np.array([oracle.entry(geo, int(i), int(j)) for i, j in ij])
        assert np.array_equal(got, G[key])


def test_library_structure_matches_golden():
    """The product's host-side tree builder (no GPU needed)."""
    lod, leaves = H.cluster_structure(G["struct_coord"])
    assert np.array_equal(lod, G["struct_lod"])
    assert np.array_equal(np.array(leaves, dtype=np.int32), G["struct_leaves"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["2dvs", "3dph", "3dnt", "2dph", "2dn", "3dht"])
def test_gpu_entries_match_golden(kind):
    prob, n, g, w, eps = case(kind, 256 if kind == "2dvs" else None)
    ij = G[f"entry_{kind}_ij"]
    for v in ("s", "n"):
        key = f"entry_{kind}_{v}"
        if key not in G:
            continue
        got = H.entry_ij(product_geometry(prob, n, g, w, v), ij[:, 0], ij[:, 1])
        ref = G[key]
        if kind == "2dvs":
            assert np.array_equal(got, ref)
        elif kind == "3dht":
            # rounding sensitivity of the free-surface correction (see
            # test_gpu_parity): absolute noise on the scale of the shear
            # self-interaction, so normal entries are measured against it too
            scale = np.max(np.abs(G[f"entry_{kind}_s"]))
            assert np.max(np.abs(got - ref)) <= 2e-6 * scale
        else:
            assert np.max(np.abs(got - ref)) <= 1e-11 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_gpu_rk_step_matches_golden():
    wl = configs.c1_2dvs(256)
    ctl = H.Ctl(256)
    lf = H.LeafMtxp(ctl, wl.geometry("s"), wl.eps_h)
    lh = H.LHp(lf, ctl, "f64")
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl)
    y0, p = wl.initial_state(lodc)
    # the host's libm (numpy log/sinh) may differ in the last bit between machines
    assert np.allclose(y0, G["rk_y0"], rtol=1e-13, atol=0)
    y0 = G["rk_y0"]
    rk = H.RK(lh, None, evlaw=0, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
    rk.set_state(y0)
    yo, ye, _ = rk.rkck(float(G["rk_h"][0]), 1.0)
    d_ref = G["rk_yout"] - y0
    assert np.linalg.norm((yo - y0) - d_ref) <= 1e-4 * np.linalg.norm(d_ref)
