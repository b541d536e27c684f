"""The ensemble (hbi_ens_*): 64 systems with their own b and dc on one pair
of FP32 H-matrices, against each member run alone through the single-system
time loop on the same operators.

Tolerance: the multi-vector product sums in another order than the
single-vector one (FP32 partial sums, ~1e-7 per product); over one
interseismic year the members' states agree within 1e-6 relative and their
slip within 1e-4."""
import numpy as np
import pytest

import hbi_gb300 as H
from hbi_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    w = configs.c2_3dph(32, 16)
    n = w.nd
    ctl_s, ctl_n = H.Ctl(n), H.Ctl(n)
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    lh_s, lh_n = H.LHp(lf_s, ctl_s, "f32"), H.LHp(lf_n, ctl_n, "f32")
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    b_in, dc_m = configs.ensemble_params(64, seed=3)
    y, vel, b, dc, p = configs.ensemble_state(w, lodc, b_in, dc_m)
    return dict(w=w, n=n, lh=(lh_s, lh_n), y=y, vel=vel, b=b, dc=dc, p=p, lodc=lodc,
                keep=(ctl_s, ctl_n, lf_s, lf_n))


@pytest.mark.parametrize("tc,tol_y,tol_s", [(False, 1e-6, 1e-4), (True, 1e-5, 1e-3)])
def test_ensemble_members_match_single_runs(setup, tc, tol_y, tol_s):
    """tc: the product on the tensor cores, factors and multipliers as BF16
    hi + lo (~16 bits each, FP32 accumulation): 1e-5 on the state."""
    S = setup
    w, p = S["w"], S["p"]
    T = 1.0 * H.YEAR
    ens = H.Ensemble(*S["lh"], S["b"], S["dc"], evlaw=w.evlaw, scale=w.scale, a=p["a"], f0=p["f0"], vpl=p["vpl"])
    if tc:
        ens.use_tensor_cores(S["keep"][2], S["keep"][3])
    ens.set_state(S["y"], S["vel"])
    st = ens.run(T, eps_r=1e-6)
    assert st["done"] == 64 and st["failed"] == 0
    ye, se, xe = ens.get_state()
    assert np.all(xe == T)
    ds = w.ds_area[S["lodc"] - 1]
    for m in (0, 17, 63):
        rk = H.RK(*S["lh"], evlaw=w.evlaw, scale=w.scale, a=p["a"], b=S["b"][:, m], dc=S["dc"][:, m], f0=p["f0"],
                  vpl=p["vpl"])
        rk.set_state(S["y"][:, m])
        cyc = H.Cycle(rk, S["vel"][:, m], ds, eps_r=1e-6)
        cs = cyc.run(t_limit=T)
        assert cs["x"] == T
        y1 = rk.get_state()
        _, s1 = cyc.fields()
        assert np.linalg.norm(ye[:, m] - y1) <= tol_y * np.linalg.norm(y1), m
        assert np.linalg.norm(se[:, m] - s1) <= tol_s * np.linalg.norm(s1), m
        cyc.close()
        rk.close()


@pytest.fixture(scope="module")
def c2_8k(oracle):
    """The c2 plane at 128 x 64 = 8,192 elements: column groups taller than
    the tensor-core kernel's 1,024-row tiles, so phase 1 also meets in
    partial sums."""
    w = configs.c2_3dph(128, 64)
    n = w.nd
    ctl_s, ctl_n = H.Ctl(n), H.Ctl(n)
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    lh_s, lh_n = H.LHp(lf_s, ctl_s, "f32"), H.LHp(lf_n, ctl_n, "f32")
    Ho = []
    for lf in (lf_s, lf_n):
        off, body = lf.body()
        Ho.append(oracle.HMatrix.from_body(n, lf.leaves(), off, body))
    tall = max(int(r[5]) for r in lf_s.leaves() if r[0] == 1)
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    b_in, dc_m = configs.ensemble_params(64, seed=5)
    y, vel, b, dc, p = configs.ensemble_state(w, lodc, b_in, dc_m)
    return dict(w=w, n=n, lf=(lf_s, lf_n), lh=(lh_s, lh_n), Ho=Ho, tall=tall, b=b, dc=dc, p=p,
                keep=(ctl_s, ctl_n))


@pytest.mark.parametrize("tc,tol", [(False, 1e-5), (True, 1e-4)])
def test_ensemble_product_against_oracle(c2_8k, tc, tol):
    """hbi_ens_product: both H-matrices applied to 64 seeded vectors, against
    the oracle's product of the same FP64 factors member by member (FP32
    store: 1e-5; tensor cores, BF16 hi + lo operands: 1e-4)."""
    S = c2_8k
    assert S["tall"] > 1024
    w, p = S["w"], S["p"]
    ens = H.Ensemble(*S["lh"], S["b"], S["dc"], evlaw=w.evlaw, scale=w.scale, a=p["a"], f0=p["f0"], vpl=p["vpl"])
    if tc:
        ens.use_tensor_cores(*S["lf"])
    X = np.random.default_rng(11).standard_normal((S["n"], 64)).astype(np.float32)
    ys, yn, _ = ens.product(X)
    for m in (0, 1, 30, 63):
        u = X[:, m].astype(np.float64)
        for y, Ho in ((ys, S["Ho"][0]), (yn, S["Ho"][1])):
            ref = Ho.matvec(u)
            assert np.linalg.norm(y[:, m] - ref) <= tol * np.linalg.norm(ref), m
    # a second product gives the same bits (fixed summation order)
    ys2, yn2, _ = ens.product(X)
    assert np.array_equal(ys, ys2) and np.array_equal(yn, yn2)
    ens.close()
