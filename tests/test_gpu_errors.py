"""Bounded waits of the product kernels end in an error status the host
reads, through the C ABI.

Every wait of the phase kernels for one of their bulk copies is bounded; a
wait that runs out sets the operator's device error word and the warp leaves
after its copies in flight have landed.  These tests make the waits run out
without anything being wrong: hbi_lh_set_wait_limit(lh, 0) gives each wait a
bound that is spent before its first probe, so every wait gives up and takes
the path of a timed-out one.  All copies are valid and are waited for (with
the default bound) before the warp leaves, so nothing faults or hangs.

Checked: the blocking product returns HBI_ERR_DEVICE, the asynchronous one
reports it through hbi_lh_check_error, the device time loop stops with
HBI_ERR_DEVICE; afterwards (default bound restored) the same operator gives
the product bit for bit again, i.e. the error word and the arrival counters
were reset.
"""
import numpy as np
import pytest

import hbi_gb300 as H
from gpu_cases import case, product_geometry
from hbi_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def operator():
    prob, n, g, w, eps = case("3dph", (64, 64))
    ctl = H.Ctl(n)
    lf = H.LeafMtxp(ctl, product_geometry(prob, n, g, w, "s"), eps)
    return n, ctl, lf


@pytest.mark.parametrize("store", ["f32", "f64"])
def test_blocking_product_reports_a_wait_that_ran_out(operator, store):
    n, ctl, lf = operator
    lh = H.LHp(lf, ctl, store)
    u = np.random.default_rng(1).standard_normal(n)
    good = lh.matvec(u)
    lh.set_wait_limit(0)
    with pytest.raises(H.HBIError) as e:
        lh.matvec(u)
    assert e.value.code == H.HBI_ERR_DEVICE
    assert b"gave up" in H.lib().hbi_last_error()
    lh.set_wait_limit(-1)
    lh.check_error()  # the blocking call already cleared the word
    assert np.array_equal(lh.matvec(u), good)
    assert np.array_equal(lh.matvec(u), good)


def test_async_product_reports_through_check_error(operator):
    import torch
    n, ctl, lf = operator
    lh = H.LHp(lf, ctl, "f32")
    st = torch.cuda.Stream()
    u = torch.randn(n, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    ref = torch.empty(n, dtype=torch.float64, device="cuda")
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    lh.matvec_dev(ref.data_ptr(), u.data_ptr(), st.cuda_stream)
    st.synchronize()
    lh.check_error()
    lh.set_wait_limit(0)
    for _ in range(3):
        lh.matvec_dev(out.data_ptr(), u.data_ptr(), st.cuda_stream)
    st.synchronize()
    with pytest.raises(H.HBIError) as e:
        lh.check_error()
    assert e.value.code == H.HBI_ERR_DEVICE
    lh.check_error()  # cleared by the first check
    lh.set_wait_limit(-1)
    lh.matvec_dev(out.data_ptr(), u.data_ptr(), st.cuda_stream)
    st.synchronize()
    lh.check_error()
    assert torch.equal(out, ref)


def test_time_loop_stops_on_a_wait_that_ran_out():
    w = configs.c1_2dvs(512)
    ctl = H.Ctl(w.nd)
    lf = H.LeafMtxp(ctl, w.geometry("s"), w.eps_h)
    lh = H.LHp(lf, ctl, "f64")
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl)
    y0, p = w.initial_state(lodc)
    ds = w.ds_area[lodc - 1]

    def loop():
        rk = H.RK(lh, None, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
        rk.set_state(y0)
        return rk, H.Cycle(rk, p["vel"], ds, eps_r=1e-6)

    lh.set_wait_limit(0)  # bound into the RK handle made next
    rk, c = loop()
    with pytest.raises(H.HBIError) as e:
        c.run(k_limit=20)
    assert e.value.code == H.HBI_ERR_DEVICE
    with pytest.raises(H.HBIError):  # a stopped loop stays stopped
        c.run(k_limit=40)
    c.close()
    rk.close()
    lh.set_wait_limit(-1)
    rk2, c2 = loop()
    st = c2.run(k_limit=20)
    assert st["stop_name"] == "klimit" and st["k"] == 20
    rk3, c3 = loop()
    c3.run(k_limit=20)
    assert np.array_equal(c2.trace(), c3.trace())


@pytest.mark.parametrize("tc", [False, True])
def test_ensemble_product_reports_a_wait_that_ran_out(tc):
    """The ensemble's product kernels (CUDA cores, and the tcgen05 kernel,
    whose roles then all leave and release tensor memory) take the bound of
    the operators they were created on: hbi_ens_product returns
    HBI_ERR_DEVICE; an ensemble created after the default bound is restored
    gives the product bit for bit."""
    w = configs.c2_3dph(32, 16)
    ctl_s, ctl_n = H.Ctl(w.nd), H.Ctl(w.nd)
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    lh = (H.LHp(lf_s, ctl_s, "f32"), H.LHp(lf_n, ctl_n, "f32"))
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    b_in, dc_m = configs.ensemble_params(64, seed=1)
    y, vel, b, dc, p = configs.ensemble_state(w, lodc, b_in, dc_m)
    X = np.random.default_rng(4).standard_normal((w.nd, 64)).astype(np.float32)

    def ensemble():
        e = H.Ensemble(*lh, b, dc, evlaw=w.evlaw, scale=w.scale, a=p["a"], f0=p["f0"], vpl=p["vpl"])
        if tc:
            e.use_tensor_cores(lf_s, lf_n)
        return e

    e = ensemble()
    ys, yn, _ = e.product(X)
    e.close()
    for o in lh:
        o.set_wait_limit(0)
    e = ensemble()
    with pytest.raises(H.HBIError) as err:
        e.product(X)
    assert err.value.code == H.HBI_ERR_DEVICE
    e.close()
    for o in lh:
        o.set_wait_limit(-1)
    e = ensemble()
    ys2, yn2, _ = e.product(X)
    e.close()
    assert np.array_equal(ys, ys2) and np.array_equal(yn, yn2)
