"""ctypes front end of the CPU oracle (oracle/_build/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py as the checker.  The product library never
imports it.  The oracle restates the reference routines listed in
oracle/hbi_oracle.h; parity against the reference binary is unpinned (no
Fortran compiler exists where this runs) and is pinned by the physics and
algorithm known answers in tests/test_oracle_pins.py.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liborc.so")

ORC_2DVS, ORC_3DPH, ORC_3DNR, ORC_3DNT, ORC_2DPH, ORC_2DN, ORC_3DHT = 1, 2, 3, 4, 5, 6, 7
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Leaf(C.Structure):
    _fields_ = [("ltmtx", C.c_int), ("kt", C.c_int), ("nstrtl", C.c_int),
                ("ndl", C.c_int), ("nstrtt", C.c_int), ("ndt", C.c_int)]


class Bemv(C.Structure):
    _fields_ = ([("problem", C.c_int), ("n", C.c_int), ("v", C.c_char), ("md", C.c_char)]
                + [(f, _dp) for f in ("xcol", "ycol", "zcol", "xel", "xer", "ang", "angd",
                                      "dsl", "dsd", "rake")]
                + [("w", C.c_double)]
                + [(f, _dp) for f in ("xs1", "xs2", "xs3", "ys1", "ys2", "ys3", "zs1", "zs2",
                                      "zs3", "ev11", "ev12", "ev13", "ev21", "ev22", "ev23",
                                      "ev31", "ev32", "ev33", "yel", "yer")])


class Rsf(C.Structure):
    _fields_ = ([("n", C.c_int), ("nmat", C.c_int), ("evlaw", C.c_int), ("backslip", C.c_int),
                 ("limitsigma", C.c_int), ("divide_ds0", C.c_int), ("ds0", C.c_double),
                 ("vref", C.c_double), ("minsig", C.c_double), ("maxsig", C.c_double)]
                + [(f, _dp) for f in ("a", "b", "dc", "f0", "vc", "taudot", "sigdot", "vplv")]
                + [("nleaf_s", C.c_int), ("leaves_s", C.POINTER(Leaf)),
                   ("off_s", C.POINTER(C.c_int64)), ("body_s", _dp),
                   ("nleaf_n", C.c_int), ("leaves_n", C.POINTER(Leaf)),
                   ("off_n", C.POINTER(C.c_int64)), ("body_n", _dp),
                   ("nthreads", C.c_int)])


def build():
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        L.orc_entry_ij.restype = C.c_double
        L.orc_znrm.restype = C.c_double
        L.orc_errmax.restype = C.c_double
        L.orc_mlp_loss_grad.restype = C.c_double
        L.orc_mlp_loss_grad_tau.restype = C.c_double
        L.orc_fill.restype = _dp
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def default_params():
    p = np.zeros(100)
    lib().orc_default_params(_p(p))
    return p


def build_structure(coord, param=None):
    """coord: (n,3) float64.  Returns (lod[n] 1-based, leaves structured array, count)."""
    coord = np.asarray(coord, dtype=np.float64)
    n = coord.shape[0]
    cf = np.asfortranarray(coord).ravel(order="F")
    lod = np.zeros(n, dtype=np.int32)
    out = C.POINTER(Leaf)()
    cnt = C.c_int(0)
    pp = _p(np.asarray(param, dtype=np.float64)) if param is not None else None
    nl = lib().orc_build_structure(n, _p(cf), pp, lod.ctypes.data_as(_ip), C.byref(out), C.byref(cnt))
    arr = np.zeros((nl, 6), dtype=np.int32)
    for i in range(nl):
        f = out[i]
        arr[i] = (f.ltmtx, f.kt, f.nstrtl, f.ndl, f.nstrtt, f.ndt)
    lib().orc_free(out)
    return lod, arr, cnt.value


class Geometry:
    """Holds numpy arrays alive behind an orc_bemv."""

    def __init__(self, problem, n, v="s", **arrays):
        self.problem, self.n = problem, n
        self.arrays = {k: np.ascontiguousarray(a, dtype=np.float64) for k, a in arrays.items()
                       if k != "w"}
        self.w = float(arrays.get("w", 0.0))
        self.set_v(v)

    def set_v(self, v):
        b = Bemv()
        b.problem, b.n, b.v, b.md = self.problem, self.n, v.encode(), b"s"
        for k, a in self.arrays.items():
            setattr(b, k, _p(a))
        b.w = self.w
        self.bemv = b
        self.v = v
        return self


def entry(g, i, j):
    return lib().orc_entry_ij(int(i), int(j), C.byref(g.bemv))


def leaves_to_struct(leaves):
    arr = (Leaf * len(leaves))()
    for i, r in enumerate(leaves):
        arr[i] = Leaf(*[int(x) for x in r])
    return arr


class HMatrix:
    """Oracle H-matrix: leaves (with kt) + body in the reference packing."""

    def __init__(self, g, lod, leaves, param=None, nthreads=1):
        if param is None:
            param = default_params()
        self.param = np.asarray(param, dtype=np.float64)
        self.n = g.n
        self.lod = np.ascontiguousarray(lod, dtype=np.int32)
        self.cleaves = leaves_to_struct(leaves)
        self.nleaf = len(leaves)
        self.off = np.zeros(self.nleaf + 1, dtype=np.int64)
        bp = lib().orc_fill(self.nleaf, self.cleaves, self.lod.ctypes.data_as(_ip), C.byref(g.bemv),
                            _p(self.param), self.off.ctypes.data_as(C.POINTER(C.c_int64)), nthreads)
        tot = int(self.off[-1])
        self.body = np.ctypeslib.as_array(bp, shape=(max(tot, 1),)).copy()[:tot]
        lib().orc_free(bp)
        self.leaves = np.array([[f.ltmtx, f.kt, f.nstrtl, f.ndl, f.nstrtt, f.ndt] for f in self.cleaves],
                               dtype=np.int32)

    @classmethod
    def from_body(cls, n, leaves, off, body):
        """Wrap factors already packed in the reference layout (e.g. exported
        from the GPU build) without running the oracle's own ACA."""
        self = cls.__new__(cls)
        self.n = n
        self.leaves = np.ascontiguousarray(leaves, dtype=np.int32)
        self.cleaves = leaves_to_struct(self.leaves)
        self.nleaf = len(self.leaves)
        self.off = np.ascontiguousarray(off, dtype=np.int64)
        self.body = np.ascontiguousarray(body, dtype=np.float64)
        return self

    def matvec(self, u, nthreads=1):
        u = np.ascontiguousarray(u, dtype=np.float64)
        au = np.zeros(self.n)
        bodyp = _p(self.body) if self.body.size else _p(np.zeros(1))
        if nthreads > 1:
            lib().orc_matvec_omp(self.n, self.nleaf, self.cleaves, self.off.ctypes.data_as(C.POINTER(C.c_int64)),
                                 bodyp, _p(u), _p(au), nthreads)
        else:
            lib().orc_matvec(self.n, self.nleaf, self.cleaves, self.off.ctypes.data_as(C.POINTER(C.c_int64)),
                             bodyp, _p(u), _p(au))
        return au

    def factors(self, ip):
        """(U ndl x kt, V ndt x kt) for a low-rank leaf, or A (ndl x ndt) for dense."""
        lt, kt, r0, ndl, c0, ndt = self.leaves[ip]
        o = int(self.off[ip])
        if lt == 1:
            V = self.body[o:o + ndt * kt].reshape(kt, ndt).T
            U = self.body[o + ndt * kt:o + (ndt + ndl) * kt].reshape(kt, ndl).T
            return U, V
        return self.body[o:o + ndl * ndt].reshape(ndl, ndt)

    def to_dense(self):
        """Dense matrix in cluster (permuted) order."""
        A = np.zeros((self.n, self.n))
        for ip in range(self.nleaf):
            lt, kt, r0, ndl, c0, ndt = self.leaves[ip]
            if lt == 1:
                U, V = self.factors(ip)
                A[r0 - 1:r0 - 1 + ndl, c0 - 1:c0 - 1 + ndt] = U @ V.T
            else:
                A[r0 - 1:r0 - 1 + ndl, c0 - 1:c0 - 1 + ndt] = self.factors(ip)
        return A


def dense_matrix(g, lod):
    """Exact dense matrix in cluster order: A[i,j] = entry(lod[i], lod[j])."""
    n = g.n
    A = np.empty((n, n))
    L = lib()
    for i in range(n):
        for j in range(n):
            A[i, j] = L.orc_entry_ij(int(lod[i]), int(lod[j]), C.byref(g.bemv))
    return A


def rows_matvec(g, lod, rows, u, nthreads=0):
    """Selected rows of the exact operator times u (cluster order):
    out[r] = sum_j entry(lod[rows[r]], lod[j]) u[j], OpenMP over the rows."""
    lod = np.ascontiguousarray(lod, dtype=np.int32)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros(len(rows))
    lib().orc_rows_matvec(C.byref(g.bemv), g.n, lod.ctypes.data_as(_ip), len(rows), rows.ctypes.data_as(_ip), _p(u),
                          _p(out), int(nthreads))
    return out


def okada(alpha, x, y, z, depth, dip, al1, al2, aw1, aw2, d1, d2, d3, fullspace=False):
    u = np.zeros(12)
    lib().orc_okada(C.c_double(alpha), C.c_double(x), C.c_double(y), C.c_double(z), C.c_double(depth),
                    C.c_double(dip), C.c_double(al1), C.c_double(al2), C.c_double(aw1), C.c_double(aw2),
                    C.c_double(d1), C.c_double(d2), C.c_double(d3), _p(u), int(fullspace))
    return u


def tdstressfs(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lam):
    s = np.zeros(6)
    P = [np.ascontiguousarray(p, dtype=np.float64) for p in (P1, P2, P3)]
    lib().orc_tdstressfs(C.c_double(X), C.c_double(Y), C.c_double(Z), _p(P[0]), _p(P[1]), _p(P[2]),
                         C.c_double(Ss), C.c_double(Ds), C.c_double(Ts), C.c_double(mu), C.c_double(lam), _p(s))
    return s


def tdstresshs(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lam):
    s = np.zeros(6)
    P = [np.ascontiguousarray(p, dtype=np.float64) for p in (P1, P2, P3)]
    lib().orc_tdstresshs(C.c_double(X), C.c_double(Y), C.c_double(Z), _p(P[0]), _p(P[1]), _p(P[2]),
                         C.c_double(Ss), C.c_double(Ds), C.c_double(Ts), C.c_double(mu), C.c_double(lam), _p(s))
    return s


def mesh_2dp(n, ds0):
    xel, xer, xcol, ds = (np.zeros(n) for _ in range(4))
    lib().orc_mesh_2dp(n, C.c_double(ds0), _p(xel), _p(xer), _p(xcol), _p(ds))
    return xel, xer, xcol, ds


def mesh_3ddip(imax, jmax, ds0, dip):
    n = imax * jmax
    xcol, ycol, zcol, angd, ang = (np.zeros(n) for _ in range(5))
    lib().orc_mesh_3ddip(imax, jmax, C.c_double(ds0), C.c_double(dip), _p(xcol), _p(ycol), _p(zcol),
                         _p(angd), _p(ang))
    return xcol, ycol, zcol, angd, ang


def evcalc(xs1, xs2, xs3, ys1, ys2, ys3, zs1, zs2, zs3):
    n = len(xs1)
    outs = [np.zeros(n) for _ in range(10)]
    ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (xs1, xs2, xs3, ys1, ys2, ys3, zs1, zs2, zs3)]
    lib().orc_evcalc(n, *[_p(a) for a in ins], *[_p(a) for a in outs])
    return outs  # ev11 ev12 ev13 ev21 ev22 ev23 ev31 ev32 ev33 ds


def cashkarp():
    a, b, c, d = np.zeros(6), np.zeros(15), np.zeros(6), np.zeros(6)
    lib().orc_cashkarp(_p(a), _p(b), _p(c), _p(d))
    return a, b, c, d


def rkqs_consts():
    c = np.zeros(4)
    lib().orc_rkqs_consts(_p(c))
    return c


class RSF:
    """Oracle rate-and-state system (derivs / rkck / rkqs)."""

    def __init__(self, n, H_s, H_n=None, evlaw=0, backslip=1, limitsigma=1, divide_ds0=0, ds0=1.0,
                 vref=float(np.float32(1e-6)), minsig=1.0, maxsig=300.0, nthreads=1, **params):
        self.keep = {}
        r = Rsf()
        r.n, r.nmat, r.evlaw, r.backslip, r.limitsigma = n, 2 if H_n is not None else 1, evlaw, backslip, limitsigma
        r.divide_ds0, r.ds0, r.vref, r.minsig, r.maxsig = divide_ds0, ds0, vref, minsig, maxsig
        for k in ("a", "b", "dc", "f0", "vc", "taudot", "sigdot", "vplv"):
            a = np.ascontiguousarray(params.get(k, np.zeros(n)), dtype=np.float64)
            self.keep[k] = a
            setattr(r, k, _p(a))
        r.nleaf_s, r.leaves_s, r.off_s, r.body_s = (H_s.nleaf, H_s.cleaves,
                                                   H_s.off.ctypes.data_as(C.POINTER(C.c_int64)), _p(H_s.body))
        if H_n is not None:
            r.nleaf_n, r.leaves_n, r.off_n, r.body_n = (H_n.nleaf, H_n.cleaves,
                                                       H_n.off.ctypes.data_as(C.POINTER(C.c_int64)), _p(H_n.body))
        r.nthreads = nthreads
        self.r, self.n = r, n
        self.H = (H_s, H_n)

    def derivs(self, y):
        d = np.zeros(3 * self.n)
        lib().orc_derivs(C.byref(self.r), C.c_double(0.0), _p(np.ascontiguousarray(y)), _p(d))
        return d

    def rkck(self, y, x, h):
        yo, ye = np.zeros(3 * self.n), np.zeros(3 * self.n)
        lib().orc_rkck(C.byref(self.r), _p(np.ascontiguousarray(y)), C.c_double(x), C.c_double(h), _p(yo), _p(ye))
        return yo, ye

    def rkqs(self, y, x, htry, eps, dtmax=1e10):
        y = np.array(y, dtype=np.float64)
        xx = C.c_double(x)
        hdid, hnext, em = C.c_double(), C.c_double(), C.c_double()
        nr = C.c_int()
        rc = lib().orc_rkqs(C.byref(self.r), _p(y), C.byref(xx), C.c_double(htry), C.c_double(eps),
                            C.c_double(dtmax), C.byref(hdid), C.byref(hnext), C.byref(em), C.byref(nr))
        return rc, y, xx.value, hdid.value, hnext.value, em.value, nr.value

    def step_update(self, y, dtdid, slip, vel):
        n = self.n
        psi, tau, sig, mu = (np.zeros(n) for _ in range(4))
        slip = np.array(slip, dtype=np.float64)
        vel = np.array(vel, dtype=np.float64)
        lib().orc_step_update(C.byref(self.r), _p(np.ascontiguousarray(y)), C.c_double(dtdid), _p(psi), _p(tau),
                              _p(sig), _p(slip), _p(vel), _p(mu))
        return psi, tau, sig, slip, vel, mu


class CycleParams(C.Structure):
    _fields_ = ([(f, C.c_double) for f in ("eps_r", "dtinit", "dtmax", "tmax", "velth", "velmax", "velmin",
                                           "dtout_inter", "dtout_co")]
                + [("interval", C.c_longlong), ("nstep", C.c_longlong)])


def cycle(rsf, y, vel, ds, nsteps, eps_r=1e-4, dtinit=1.0, dtmax=1e10, tmax_yr=1e4,
          velth=float(np.float32(1e-2)), velmax=1e7, velmin=1e-20, dtout_yr=1.0, dtout_co=1000.0, interval=0,
          nstep=1000000, max_events=10000):
    """The time loop of main_LH.f90:1217-1438 (no files).  Returns (stop,
    records[k, x, hdid, errmax, nrjct, mvel, loc, meanslip, meanmu, maxnorm,
    minnorm, outfield], events[id, k, onset, moment, hypoloc, x], y, vel, slip)."""
    year = 365 * 24 * 3600.0
    cp = CycleParams(eps_r, dtinit, dtmax, tmax_yr * year, velth, velmax, velmin, dtout_yr * year, dtout_co,
                     interval, nstep)
    n = rsf.n
    y = np.array(y, dtype=np.float64)
    vel = np.array(vel, dtype=np.float64)
    slip = np.zeros(n)
    ds = np.ascontiguousarray(ds, dtype=np.float64)
    rec = np.zeros((nsteps, 12))
    ev = np.zeros((max_events, 6))
    nrec, nev = C.c_longlong(), C.c_int()
    stop = lib().orc_cycle(C.byref(rsf.r), C.byref(cp), _p(y), _p(vel), _p(slip), _p(ds), C.c_longlong(nsteps),
                           _p(rec), C.byref(nrec), _p(ev), C.c_int(max_events), C.byref(nev))
    return stop, rec[:nrec.value], ev[:min(nev.value, max_events)], y, vel, slip


def mlp_loss_grad(nin, h, params, x, target, tau=-1.0):
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    g = np.zeros_like(params)
    out = np.zeros(len(target), dtype=np.float32)
    fp = C.POINTER(C.c_float)
    loss = lib().orc_mlp_loss_grad_tau(nin, h, len(target), params.ctypes.data_as(fp), x.ctypes.data_as(fp),
                                       target.ctypes.data_as(fp), g.ctypes.data_as(fp), out.ctypes.data_as(fp),
                                       C.c_double(tau))
    return loss, g, out
