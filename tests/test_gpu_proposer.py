"""The learned step-size proposer: its training kernels against the oracle's
forward/backward restatement, and what the trained network gains over the
rkqs controller alone on the 2D antiplane cycle.

Tolerances: loss and gradients of the GPU kernels (float32 sums) within 2e-4
relative of the oracle (double sums), per parameter block.  The A/B run: the
learned controller must reject a smaller fraction of attempts and spend fewer
attempts per simulated year than rkqs alone, with the event onset times and
the mean slip of each event within 1e-3 relative of the rkqs run.
"""
import numpy as np
import pytest

import hbi_gb300 as H
from hbi_gb300 import configs, proposer

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tau", [None, 0.2])
def test_mlp_gradients_match_oracle(oracle, tau):
    """Squared error, and the pinball loss of quantile 0.2 (targets shifted so
    that no residual sits near the loss's kink)."""
    nin, hid, B = 6, 64, 512
    rng = np.random.default_rng(3)
    m = H.MLP(nin, hid, batch_max=B)
    p = m.init(seed=4)
    p[: hid * nin + hid] += 0.05 * rng.standard_normal(hid * nin + hid).astype(np.float32)  # nonzero biases
    m.set_params(p)
    m.set_loss(tau)
    x = rng.standard_normal((B, nin)).astype(np.float32)
    t = rng.standard_normal(B).astype(np.float32) + (0.0 if tau is None else 3.0)
    loss, g, out = m.loss_grad(x, t)
    loss_o, g_o, out_o = oracle.mlp_loss_grad(nin, hid, p, x, t, -1.0 if tau is None else tau)
    assert abs(loss - loss_o) <= 2e-4 * abs(loss_o)
    assert np.allclose(out, out_o, rtol=2e-4, atol=2e-5)
    o = 0
    for size in (hid * nin, hid, hid * hid, hid, hid, 1):
        gb, gbo = g[o:o + size], g_o[o:o + size]
        assert np.linalg.norm(gb - gbo) <= 2e-4 * np.linalg.norm(gbo) + 1e-7, o
        o += size


def test_mlp_training_reduces_loss():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((8192, 6)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2]).astype(np.float32)
    m = H.MLP(6, 64, batch_max=1024)
    m.init(seed=1)
    hist = m.train(x, t, epochs=20, batch=512, lr=3e-3, seed=2)
    assert hist[-1] < 0.1 * hist[0]
    pred = m.predict(x[:100])
    _, _, out = m.loss_grad(x[:100], t[:100])
    assert np.allclose(pred, out, rtol=1e-6, atol=1e-6)


def _system(n=1024):
    w = configs.c1_2dvs(n)
    ctl = H.Ctl(n)
    lf = H.LeafMtxp(ctl, w.geometry("s"), w.eps_h)
    lh = H.LHp(lf, ctl, "f64")
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl)
    y0, p = w.initial_state(lodc)
    return dict(lh=lh, y0=y0, p=p, ds=w.ds_area[lodc - 1], keep=(ctl, lf))


def _run(S, tyr, w=None):
    p = S["p"]
    rk = H.RK(S["lh"], None, evlaw=0, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
    rk.set_state(S["y0"])
    c = H.Cycle(rk, p["vel"], S["ds"], eps_r=1e-6, tmax_yr=1500.0)
    if w is not None:
        c.set_proposer(w)
    st = c.run(t_limit=tyr * H.YEAR)
    return st, c.trace(), c.events()


def test_learned_proposer_gains_over_rkqs():
    S = _system()
    # training data: the rkqs controller's own trace of the first 300 years
    _, tr_train, _ = _run(S, 300.0)
    X, T = proposer.training_set(tr_train)
    assert len(T) > 5000
    w, hist = proposer.train(X, T, epochs=30)
    assert hist[-1] < hist[0]
    # A/B over 600 years (twice the training window)
    st_c, tr_c, ev_c = _run(S, 600.0)
    st_l, tr_l, ev_l = _run(S, 600.0, w)
    rej_c = st_c["rejected"] / st_c["attempts"]
    rej_l = st_l["rejected"] / st_l["attempts"]
    assert rej_l < rej_c, (rej_l, rej_c)
    assert st_l["attempts"] < st_c["attempts"], (st_l["attempts"], st_c["attempts"])
    assert len(ev_l) == len(ev_c) and len(ev_c) >= 3
    for a, b in zip(ev_l, ev_c):
        assert abs(a["onset"] - b["onset"]) <= 1e-3 * b["onset"]
        assert abs(a["moment"] - b["moment"]) <= 1e-3 * abs(b["moment"])


def test_mixed_form_passes_the_catalogue_gate():
    """The accuracy gate of the mixed form at small size: c1 (1,024
    elements) over 600 years, the plain form (FP64 factors, rkqs) against
    FP32 factors with the proposer trained on the plain run's trace; the
    catalogues and slip fields compared by hbi_gb300.catalogue (earthquakes
    paired one to one within 1e-3 in onset and slip, every event matched,
    slip field within 1e-3)."""
    from hbi_gb300.catalogue import catalogue_gate
    S = _system()
    p = S["p"]

    def run(lh, w=None):
        rk = H.RK(lh, None, evlaw=0, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
        rk.set_state(S["y0"])
        c = H.Cycle(rk, p["vel"], S["ds"], eps_r=1e-6, tmax_yr=1500.0)
        if w is not None:
            c.set_proposer(w)
        st = c.run(t_limit=600.0 * H.YEAR)
        return dict(st=st, trace=c.trace(), events=c.events(), slip=c.fields()[1])

    plain = run(S["lh"])
    X, T = proposer.training_set(plain["trace"])
    w, _ = proposer.train(X, T, epochs=30)
    ctl, lf = S["keep"]
    mixed = run(H.LHp(lf, ctl, "f32"), w)
    g = catalogue_gate(plain, mixed)
    assert g["earthquakes"][0] >= 5, g
    assert g["pass"], g["failures"]
