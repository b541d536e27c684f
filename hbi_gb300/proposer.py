"""Learned step-size proposer: training data from the solver's own traces,
training on the GPU (hbi_mlp_* kernels) and packing for the time loop.

After step k is accepted, the time loop feeds the MLP seven numbers known at
that moment (the features of hbi_cycle.cu's proposer_features): log10 of this
step's error and of the previous one, the step growth log10(h_k/h_{k-1}), the
slip-rate trend log10(V_{k-1}/V_{k-2}) of the monitors, the rejections of
this step, rkqs's own growth log10(h_next/h_k) and log10 V_{k-1}.  The network
answers d = log10(h_try / rkqs h_next) for step k+1, clamped to [lo, hi].
With hi = 0 the proposer only ever shortens rkqs's step: it acts where it
foresees a rejection (the error growing faster than rkqs assumes, as when a
rupture nucleates) and leaves rkqs's step alone elsewhere.

The training target comes from the trace of a run: the first attempt of step
k+1 was tried with h1 and gave error e1; Cash-Karp's error scales with h**5,
so h* = h1 (e_target/e1)**0.2 would have given e_target, and the label is
d* = log10(h*/h_next).  e_target < 1 keeps a margin below the rejection
threshold; the rkqs error test still judges every attempt.
"""
import numpy as np

from . import MLP, proposer_size

E_TARGET = 0.5
LO, HI = -1.0, 0.0
TINY = 1e-30


def _l10(v):
    return np.log10(np.maximum(v, TINY))


def features(e, e_prev, h, h_prev, v1, v2, nrjct, hnext):
    """The seven inputs, as the device computes them (float32)."""
    f = np.stack([_l10(e), _l10(e_prev), _l10(h) - _l10(h_prev), _l10(v1) - _l10(v2), np.asarray(nrjct, float),
                  _l10(hnext) - _l10(h), _l10(v1)], axis=-1)
    return f.astype(np.float32)


def training_set(trace, e_target=E_TARGET):
    """(X, T) from a time-loop trace (rows: k, x, h, errmax, accepted, mvel,
    hnext, nrjct per attempt)."""
    tr = np.asarray(trace)
    rows = np.nonzero(tr[:, 4] == 1)[0]
    if len(rows) < 4:
        return np.zeros((0, 6), np.float32), np.zeros(0, np.float32)
    A = tr[rows]
    j = np.arange(2, len(rows) - 1)           # step j with a successor attempt
    nxt = rows[j] + 1
    keep = nxt < len(tr)
    j, nxt = j[keep], nxt[keep]
    h1, e1 = tr[nxt, 2], tr[nxt, 3]
    ok = np.isfinite(e1) & (e1 > 0) & (A[j, 6] > 0)
    j, h1, e1 = j[ok], h1[ok], e1[ok]
    X = features(A[j, 3], A[j - 1, 3], A[j, 2], A[j - 1, 2], A[j - 1, 5], A[j - 2, 5], A[j, 7], A[j, 6])
    T = (_l10(h1) - _l10(A[j, 6]) + 0.2 * (np.log10(e_target) - _l10(e1))).astype(np.float32)
    return X, T


def pack(params, mean, sd, lo=LO, hi=HI):
    """Weight vector of hbi_cycle_set_proposer: MLP parameters, input
    standardisation, output clamp."""
    nin, hid, nf = proposer_size()
    w = np.concatenate([np.asarray(params, np.float32), np.asarray(mean, np.float32), np.asarray(sd, np.float32),
                        np.array([lo, hi], np.float32)])
    assert w.size == nf, (w.size, nf)
    return w


def train(X, T, epochs=40, batch=1024, lr=2e-3, seed=0, min_steps=3000, tau=None, lo=LO, hi=HI):
    """Fit the proposer on the GPU; returns (weight vector, loss per epoch).
    Small traces get smaller batches and more epochs, so that every fit takes
    at least `min_steps` Adam steps.  tau: None fits the mean of the label
    (squared error); 0 < tau < 1 fits its tau-quantile (pinball loss), a
    proposal that the ideal step exceeds with probability 1 - tau.  lo, hi:
    the clamp of the proposal d."""
    nin, hid, _ = proposer_size()
    batch = int(min(batch, max(64, len(T) // 8)))
    epochs = int(max(epochs, -(-min_steps * batch // max(1, len(T)))))
    mean = X.mean(axis=0)
    sd = X.std(axis=0)
    sd = np.where(sd > 1e-6, sd, 1.0)
    Xs = ((X - mean) / sd).astype(np.float32)
    m = MLP(nin, hid, batch_max=max(batch, 64))
    m.init(seed)
    m.set_loss(tau)
    hist = m.train(Xs, T, epochs=epochs, batch=min(batch, len(T)), lr=lr, seed=seed)
    w = pack(m.params(), mean, sd, lo, hi)
    m.close()
    return w, hist
