"""The device-resident time loop (hbi_cycle_*) against the oracle's
restatement of main_LH.f90:1217-1438, through the C ABI.

Both loops run the 2D antiplane system with b tapering below 15 km on the
same FP64 factors, from the same seeded initial state, through the first
earthquake.  Tolerances:
  * the first 200 steps: times and step sizes within 1e-6 relative, the
    rejection count of every step equal.  The products differ only in
    summation order (~1e-15 relative), but the error estimate yerr is a
    difference of stage sums that cancels to ~1e-6 of the state, so errmax,
    and through errmax**-0.2 the next step size, carry ~1e-9..1e-8 relative
    differences that accumulate over the steps;
  * the first event: onset time within 1e-6 relative, hypocentre equal, mean
    slip within 1e-6 relative (the nucleation amplifies the round-off of the
    steps before it); the mean friction after the event within 1e-5;
  * the loop is deterministic: a run split by a step limit gives the same
    records as one run, bit for bit; a time limit is landed on exactly.
"""
import os

import numpy as np
import pytest

import hbi_gb300 as H
from hbi_gb300 import configs

pytestmark = pytest.mark.gpu

N = 512
STEPS = 3400


@pytest.fixture(scope="module")
def system(oracle):
    w = configs.c1_2dvs(N)
    ctl = H.Ctl(N)
    lf = H.LeafMtxp(ctl, w.geometry("s"), w.eps_h)
    lh = H.LHp(lf, ctl, "f64")
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl)
    y0, p = w.initial_state(lodc)
    ds = w.ds_area[lodc - 1]
    off, body = lf.body()
    Ho = oracle.HMatrix.from_body(N, lf.leaves(), off, body)
    R = oracle.RSF(N, Ho, evlaw=0, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vplv=p["vpl"])
    return dict(w=w, lh=lh, y0=y0, p=p, ds=ds, R=R, keep=(ctl, lf))


def _cycle(S, **kw):
    p = S["p"]
    rk = H.RK(S["lh"], None, evlaw=0, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
    rk.set_state(S["y0"])
    kw.setdefault("eps_r", 1e-6)
    kw.setdefault("tmax_yr", 1500.0)
    return H.Cycle(rk, p["vel"], S["ds"], **kw)


@pytest.fixture(scope="module")
def oracle_run(oracle, system):
    S = system
    return oracle.cycle(S["R"], S["y0"], S["p"]["vel"], S["ds"], STEPS, eps_r=1e-6, tmax_yr=1500.0)


def test_cycle_follows_oracle_loop(system, oracle_run):
    stop_o, rec, ev_o, y_o, vel_o, slip_o = oracle_run
    assert len(ev_o) >= 1, "the comparison window must contain an event"
    c = _cycle(system)
    st = c.run(k_limit=STEPS)
    assert st["stop_name"] == "klimit" and st["k"] == STEPS
    tr = c.trace()
    acc = tr[tr[:, 4] == 1]
    assert len(acc) == STEPS
    # per-step controller decisions over the first 200 steps
    m = 200
    assert np.array_equal(acc[:m, 0], rec[:m, 0])
    assert np.allclose(acc[:m, 1], rec[:m, 1], rtol=1e-6, atol=0)     # x
    assert np.allclose(acc[:m, 2], rec[:m, 2], rtol=1e-6, atol=0)     # accepted h
    assert np.array_equal(acc[:m, 7], rec[:m, 4])                     # nrjct
    assert np.allclose(acc[:m, 5], rec[:m, 5], rtol=1e-6, atol=0)     # max slip rate
    # the first event
    ev_g = c.events()
    assert len(ev_g) >= 1
    e_g, e_o = ev_g[0], ev_o[0]
    assert e_g["id"] == int(e_o[0]) == 1
    assert e_g["hypoloc"] == int(e_o[4])
    assert abs(e_g["onset"] - e_o[2]) <= 1e-6 * e_o[2]
    assert abs(e_g["moment"] - e_o[3]) <= 1e-6 * abs(e_o[3])
    # monitors of the last step, after the event has amplified the round-off
    assert abs(st["meanmu"] - rec[-1, 8]) <= 1e-5 * abs(rec[-1, 8])
    assert st["rejected"] == int(tr[:, 4].size - STEPS)


def test_cycle_split_runs_are_identical(system):
    a = _cycle(system)
    a.run(k_limit=300)
    b = _cycle(system, inflight=1)
    b.run(k_limit=120)
    b.run(k_limit=300)
    ta, tb = a.trace(), b.trace()
    assert ta.shape == tb.shape
    assert np.array_equal(ta, tb)
    va, sa = a.fields()
    vb, sb = b.fields()
    assert np.array_equal(va, vb) and np.array_equal(sa, sb)


def test_cycle_lands_on_time_limits(system):
    c = _cycle(system)
    for t in (0.5 * H.YEAR, 2.0 * H.YEAR):
        st = c.run(t_limit=t)
        assert st["stop_name"] == "tlimit"
        assert st["x"] == t


def test_cycle_writes_reference_files(system, tmp_path):
    out = str(tmp_path)
    c = _cycle(system, outdir=out, number=7, interval=100)
    st = c.run(k_limit=400)
    c.close()
    mon = open(os.path.join(out, "monitor7.dat")).read().splitlines()
    assert len(mon) == 401
    # '(i7,f19.4,7e16.5,i4,f16.4)'
    assert all(len(l) == 7 + 19 + 7 * 16 + 4 + 16 for l in mon)
    assert int(mon[0][:7]) == 0 and int(mon[-1][:7]) == 400
    assert "E" in mon[1][26:42]
    times = open(os.path.join(out, "time7.dat")).read().splitlines()
    assert len(times) >= 1 + 4 and all(len(l) == 26 for l in times)
    ks = [int(l[:7]) for l in times]
    assert ks[0] == 0 and {100, 200, 300, 400} <= set(ks)
    for f in ("vel", "slip", "sigma", "tau"):
        assert os.path.getsize(os.path.join(out, f"{f}7.dat")) == 8 * N * len(times)
    vel = np.fromfile(os.path.join(out, "vel7.dat")).reshape(len(times), N)
    assert np.array_equal(vel[0], system["p"]["vel"])
    assert st["k"] == 400


def test_zero_proposer_is_the_classic_controller(system):
    nin, hid, nf = H.proposer_size()
    w = np.zeros(nf, dtype=np.float32)
    w[nf - 2 * nin - 2 + nin: nf - 2] = 1.0  # sd = 1
    w[nf - 2], w[nf - 1] = -1.0, 0.5         # clamp
    a = _cycle(system)
    a.run(k_limit=250)
    b = _cycle(system)
    b.set_proposer(w)
    b.run(k_limit=250)
    assert np.array_equal(a.trace(), b.trace())
    # a proposer that always halves the rkqs proposal takes more steps
    w[nf - 2 * nin - 3] = np.log10(0.5)      # b3
    c = _cycle(system)
    c.set_proposer(w)
    c.run(k_limit=250)
    assert c.trace()[-1, 1] < a.trace()[-1, 1]


def test_cycle_restart_continues_a_run(system, tmp_path):
    """A run stopped at step 100 and restarted from its own files
    (main_LH.f90:836-957) reaches the same state at a later time as an
    uninterrupted run (before the first earthquake).  The restart point
    carries x to 1e-4 s and the next step to 5 digits (the monitor file's
    formats) and psi is rebuilt from V, so the two runs take different steps
    at the RK tolerance: the states agree to 1e-5, the slip to 1e-4."""
    out = str(tmp_path)
    a = _cycle(system, outdir=out, number=3, interval=50)
    sa = a.run(k_limit=100)  # about 12.7 years: interseismic
    a.close()
    assert sa["x"] < 16.0 * H.YEAR
    T = 16.0 * H.YEAR  # the nucleation starts after 21 years
    p = system["p"]
    rk = H.RK(system["lh"], None, evlaw=0, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
    b = H.Cycle(rk, p["vel"], system["ds"], eps_r=1e-6, tmax_yr=1500.0, outdir=out, number=3, interval=100,
                restart=True)
    sb = b.run(t_limit=T)
    yb = rk.get_state()
    _, slip_b = b.fields()
    c = _cycle(system)
    sc = c.run(t_limit=T)
    yc = c.rk.get_state()
    _, slip_c = c.fields()
    assert sb["x"] == T and sc["x"] == T
    assert np.linalg.norm(yb - yc) <= 1e-5 * np.linalg.norm(yc)
    assert np.linalg.norm(slip_b - slip_c) <= 1e-4 * np.linalg.norm(slip_c)
    mon = open(os.path.join(out, "monitor3.dat")).read().splitlines()
    ks = [int(l[:7]) for l in mon]
    assert ks[:101] == list(range(101)) and ks[101] == 101 and len(set(ks)) == len(ks)
    # a limit already reached runs nothing
    assert b.run(t_limit=T)["stop_name"] == "tlimit"


@pytest.mark.parametrize("kind", ["2dph", "3dht"])
def test_cycle_with_two_matrices_follows_oracle(oracle, kind):
    """The loop on the newer problem kinds -- 2D edge dislocations in a half
    space and triangles in a half space -- with both the shear and the normal
    H-matrix (sigma evolves), against the oracle's loop on the same FP64
    factors: the interseismic steps (80 for 2dph, whose patch starts to
    nucleate near step 105; 150 for 3dht), times and step sizes within 1e-6
    relative, rejection counts equal."""
    from gpu_cases import case, product_geometry
    prob, n, g, w, eps = case(kind)
    lhs, keep = [], []
    Ho = []
    for v in ("s", "n"):
        ctl = H.Ctl(n)
        lf = H.LeafMtxp(ctl, product_geometry(prob, n, g, w, v), eps)
        lhs.append(H.LHp(lf, ctl, "f64"))
        off, body = lf.body()
        Ho.append(oracle.HMatrix.from_body(n, lf.leaves(), off, body))
        keep.append((ctl, lf))
    ndc, lodc = H.HACApK_gen_lattice_vector(keep[0][0])
    rng = np.random.default_rng(5)
    idx = lodc - 1
    mid = np.abs(np.arange(n) - n / 2) < 0.3 * n
    a = np.full(n, 0.01)
    b = np.where(mid, 0.015, 0.006)[idx]
    dc = np.full(n, 0.01)
    f0 = np.full(n, 0.6)
    vpl = np.full(n, 1e-9)
    vel = (1e-9 * (1 + 0.01 * rng.uniform(-1, 1, n)))[idx]
    sig = np.full(n, 50.0)
    vref = float(np.float32(1e-6))
    psi_ss = f0 - b * np.log(vel / vref)
    tau = a * sig * np.arcsinh(vel / (2 * vref) * np.exp(psi_ss / a))
    psi = a * np.log(2 * vref / vel * np.sinh(tau / sig / a))
    y0 = np.empty(3 * n)
    y0[0::3], y0[1::3], y0[2::3] = psi, tau, sig
    evlaw = 1 if kind == "3dht" else 0
    ds = np.full(n, 1.0)
    steps = 80 if kind == "2dph" else 150
    R = oracle.RSF(n, Ho[0], Ho[1], evlaw=evlaw, a=a, b=b, dc=dc, f0=f0, vplv=vpl)
    stop_o, rec, ev_o, y_o, vel_o, slip_o = oracle.cycle(R, y0, vel, ds, steps, eps_r=1e-6, tmax_yr=1500.0)
    rk = H.RK(lhs[0], lhs[1], evlaw=evlaw, a=a, b=b, dc=dc, f0=f0, vpl=vpl)
    rk.set_state(y0)
    c = H.Cycle(rk, vel, ds, eps_r=1e-6, tmax_yr=1500.0)
    st = c.run(k_limit=steps)
    assert st["k"] == steps and len(rec) == steps
    tr = c.trace()
    acc = tr[tr[:, 4] == 1]
    assert np.allclose(acc[:steps, 1], rec[:steps, 1], rtol=1e-6, atol=0)   # x
    assert np.allclose(acc[:steps, 2], rec[:steps, 2], rtol=1e-6, atol=0)   # accepted h
    assert np.array_equal(acc[:steps, 7], rec[:steps, 4])                   # nrjct
    y = rk.get_state()
    assert np.linalg.norm(y - y_o) <= 1e-6 * np.linalg.norm(y_o)
    c.close()
    rk.close()
