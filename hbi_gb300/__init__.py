"""hbi_gb300 -- GB300 (sm_103a) implementation of HBI's per-step hot path.

Host-side mirror of the HACApK entry points the HBI driver calls
(HACApK_init / _generate / _construct_LH / _gen_lattice_vector /
_adot_lattice_hyp, and the derivs/rkck/rkqs loop of main_LH.f90), bound to
the C ABI in include/hbi_gpu.h through ctypes.  The library is built in-tree
by hbi_gb300/_build.py; importing this module on a machine without it, or
calling a compute entry point without a GPU, raises HBIError -- there is no
CPU fallback.
"""
import atexit
import ctypes as C
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libhbigpu.so")

HBI_2DVS, HBI_3DPH, HBI_3DNR, HBI_3DNT, HBI_2DPH, HBI_2DN, HBI_3DHT = 1, 2, 3, 4, 5, 6, 7
STORE_F64, STORE_F32, STORE_BF16 = 0, 1, 2
STORE_NAMES = {"f64": STORE_F64, "f32": STORE_F32, "bf16": STORE_BF16}
HBI_ERR_CONVERGE = -5
HBI_ERR_LIMIT = -6
HBI_ERR_DEVICE = -7

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)

# exported symbols of include/hbi_gpu.h (checked by the CPU test suite)
EXPORTS = [
    "hbi_last_error", "hbi_version", "hbi_init", "hbi_param_set", "hbi_param_get", "hbi_finalize",
    "hbi_generate", "hbi_free_leafmtxp", "hbi_construct_lh", "hbi_free_lh", "hbi_gen_lattice_vector",
    "hbi_adot_lattice_hyp", "hbi_adot_lattice_hyp_dev", "hbi_entry_ij", "hbi_get_lod", "hbi_leaf_count",
    "hbi_get_leaves", "hbi_get_body", "hbi_lh_info", "hbi_rk_create", "hbi_rk_free", "hbi_rk_set_state",
    "hbi_rk_get_state", "hbi_derivs", "hbi_rkck", "hbi_rkqs", "hbi_rk_launches_per_attempt",
    "hbi_cluster_structure", "hbi_rk_stream", "hbi_rk_attempt_async", "hbi_set_device",
    "hbi_adot_lattice_hyp_phase_dev", "hbi_lh_phase_bytes", "hbi_adot_lattice_hyp_noalloc",
    "hbi_cycle_create", "hbi_cycle_run", "hbi_cycle_fields", "hbi_cycle_events", "hbi_cycle_trace",
    "hbi_cycle_free", "hbi_cycle_set_proposer", "hbi_cycle_proposer_size",
    "hbi_mlp_create", "hbi_mlp_free", "hbi_mlp_set_params", "hbi_mlp_get_params", "hbi_mlp_loss_grad",
    "hbi_mlp_train", "hbi_mlp_predict", "hbi_plan_emulate", "hbi_umma_probe",
    "hbi_ens_create", "hbi_ens_free", "hbi_ens_set_state", "hbi_ens_get_state", "hbi_ens_run",
    "hbi_tc_plan_emulate", "hbi_ens_use_tensor_cores", "hbi_ens_product", "hbi_cycle_restart", "hbi_restart_point",
    "hbi_plan_warp_schedule", "hbi_plan_block_schedule", "hbi_lh_check_error", "hbi_lh_set_wait_limit", "hbi_rk_check_error",
    "hbi_stream_shapes", "hbi_lh_tuning", "hbi_autotune_select", "hbi_lh_set_shapes",
    "hbi_partition_leaves", "hbi_construct_lh_part", "hbi_mlp_set_loss",
]


def set_device(device):
    """Bind subsequent handles of this thread to CUDA device `device`."""
    _check(lib().hbi_set_device(int(device)), "hbi_set_device")


class HBIError(RuntimeError):
    pass


class Bemv(C.Structure):
    """hbi_bemv == st_HACApK_calc_entry (m_HACApK_calc_entry_ij.f90:7-19)."""
    _fields_ = ([("problem", C.c_int), ("nd", C.c_int), ("v", C.c_char), ("md", C.c_char)]
                + [(f, _dp) for f in ("xcol", "ycol", "zcol", "xel", "xer", "ang", "angd", "dsl", "dsd", "rake")]
                + [("w", C.c_double)]
                + [(f, _dp) for f in ("xs1", "xs2", "xs3", "ys1", "ys2", "ys3", "zs1", "zs2", "zs3", "ev11",
                                      "ev12", "ev13", "ev21", "ev22", "ev23", "ev31", "ev32", "ev33",
                                      "yel", "yer")])


class CycleParams(C.Structure):
    """hbi_cycle_params: the time-loop controls of main_LH.f90 (:133-160, :330-332)."""
    _fields_ = ([(f, C.c_double) for f in ("eps_r", "dtinit", "dtmax", "tmax", "velth", "velmax", "velmin",
                                           "dtout_inter", "dtout_co", "rigid")]
                + [("nstep", C.c_longlong), ("interval", C.c_longlong), ("number", C.c_int), ("inflight", C.c_int),
                   ("pad0", C.c_int), ("pad1", C.c_int), ("outdir", C.c_char_p)])


class CycleStatus(C.Structure):
    _fields_ = ([("k", C.c_longlong), ("attempts", C.c_longlong), ("rejected", C.c_longlong)]
                + [(f, C.c_double) for f in ("x", "hnext", "errmax", "dtdid", "mvel", "meanslip", "meanmu",
                                             "maxnorm", "minnorm")]
                + [(f, C.c_int) for f in ("nrjct", "events", "slipping", "stop")]
                + [("wall_s", C.c_double)])

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Event(C.Structure):
    _fields_ = [("id", C.c_int), ("hypoloc", C.c_int), ("k", C.c_longlong), ("onset", C.c_double),
                ("end", C.c_double), ("moment", C.c_double), ("mw", C.c_double)]


STOP_NAMES = {0: "none", 1: "tmax", 2: "velmax", 3: "velmin", 4: "klimit", 5: "underflow", 6: "tlimit", 7: "device"}
YEAR = 365 * 24 * 3600.0


class RsfParams(C.Structure):
    _fields_ = ([("ncell", C.c_int), ("evlaw", C.c_int), ("backslip", C.c_int), ("limitsigma", C.c_int),
                 ("vref", C.c_double), ("minsig", C.c_double), ("maxsig", C.c_double),
                 ("scale_s", C.c_double), ("scale_n", C.c_double)]
                + [(f, _dp) for f in ("a", "b", "dc", "f0", "taudot", "sigdot", "vpl")])


_lib = None
_live = weakref.WeakValueDictionary()  # id -> handle owner, for ordered teardown at exit
_closed = False


def _register(obj, rank):
    obj._rank = rank
    _live[id(obj)] = obj


@atexit.register
def _teardown():
    """Free live handles before the CUDA runtime goes away: time loops first,
    then RK states, operators, filled H-matrices and control blocks."""
    global _closed
    for rank in (0, 1, 2, 3, 4):
        for obj in list(_live.values()):
            if getattr(obj, "_rank", -1) == rank:
                obj.close()
    _closed = True


def lib():
    """Load libhbigpu.so (built by hbi_gb300._build.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise HBIError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        L.hbi_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc, what):
    if rc != 0:
        msg = lib().hbi_last_error().decode(errors="replace")
        err = HBIError(f"{what} failed ({rc}): {msg}")
        err.code = rc
        raise err


def _p(a):
    return a.ctypes.data_as(_dp)


class Geometry:
    """Keeps numpy arrays alive behind an hbi_bemv (global element order)."""

    def __init__(self, problem, nd, v="s", w=0.0, **arrays):
        self.problem, self.nd, self.w = problem, nd, float(w)
        self.arrays = {k: np.ascontiguousarray(a, dtype=np.float64) for k, a in arrays.items()}
        for k, a in self.arrays.items():
            if a.shape != (nd,):
                raise ValueError(f"geometry array {k} has shape {a.shape}, expected ({nd},)")
        self.set_v(v)

    def set_v(self, v):
        b = Bemv()
        b.problem, b.nd, b.v, b.md, b.w = self.problem, self.nd, v.encode(), b"s", self.w
        for k, a in self.arrays.items():
            setattr(b, k, _p(a))
        self.bemv, self.v = b, v
        return self

    def coord(self):
        z = np.zeros(self.nd)
        x = self.arrays.get("xcol", z)
        y = self.arrays.get("ycol", z)
        zz = self.arrays.get("zcol", z)
        return np.asfortranarray(np.stack([x, y, zz], 1))


class Ctl:
    """st_HACApK_lcontrol: HACApK_init (m_HACApK_base.f90:246-345)."""

    def __init__(self, nd):
        self.h = C.c_void_p()
        _check(lib().hbi_init(int(nd), C.byref(self.h)), "hbi_init")
        self.nd = nd
        _register(self, 4)

    @property
    def param(self):
        p = np.zeros(100)
        _check(lib().hbi_param_get(self.h, _p(p)), "hbi_param_get")
        return p

    @param.setter
    def param(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        _check(lib().hbi_param_set(self.h, _p(p)), "hbi_param_set")

    def lod(self):
        a = np.zeros(self.nd, dtype=np.int32)
        _check(lib().hbi_get_lod(self.h, a.ctypes.data_as(_ip)), "hbi_get_lod")
        return a

    def close(self):
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_finalize(self.h)
        self.h = None

    def __del__(self):
        self.close()


class LeafMtxp:
    """st_HACApK_leafmtxp: result of HACApK_generate."""

    def __init__(self, ctl, geom, ztol):
        self.ctl, self.h = ctl, C.c_void_p()
        coord = geom.coord().ravel(order="F")
        _check(lib().hbi_generate(C.byref(self.h), C.byref(geom.bemv), ctl.h, _p(coord), C.c_double(ztol)),
               "hbi_generate")
        _register(self, 3)

    def leaves(self):
        n, km = C.c_int(), C.c_int()
        _check(lib().hbi_leaf_count(self.h, C.byref(n), C.byref(km)), "hbi_leaf_count")
        a = np.zeros((n.value, 6), dtype=np.int32)
        _check(lib().hbi_get_leaves(self.h, a.ctypes.data_as(_ip)), "hbi_get_leaves")
        return a

    def body(self):
        nl = len(self.leaves())
        off = np.zeros(nl + 1, dtype=np.int64)
        _check(lib().hbi_get_body(self.h, off.ctypes.data_as(_i64p), None), "hbi_get_body")
        body = np.zeros(max(int(off[-1]), 1))
        _check(lib().hbi_get_body(self.h, off.ctypes.data_as(_i64p), _p(body)), "hbi_get_body")
        return off, body[:int(off[-1])]

    def close(self):
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_free_leafmtxp(self.h)
        self.h = None

    def __del__(self):
        self.close()


class LHp:
    """st_HACApK_LHp: the lattice matvec operator (HACApK_construct_LH)."""

    def __init__(self, lf, ctl, storage=STORE_F64, owner=None, rank=0):
        """owner (per leaf, from partition_leaves) and rank: the operator of
        one rank's leaves (its product is that rank's partial product)."""
        if isinstance(storage, str):
            storage = STORE_NAMES[storage]
        self.ctl, self.h, self.storage = ctl, C.c_void_p(), storage
        if owner is None:
            _check(lib().hbi_construct_lh(C.byref(self.h), lf.h, ctl.h, int(storage)), "hbi_construct_lh")
        else:
            self._owner = np.ascontiguousarray(owner, dtype=np.int32)
            _check(lib().hbi_construct_lh_part(C.byref(self.h), lf.h, ctl.h, int(storage),
                                               self._owner.ctypes.data_as(_ip), int(rank)), "hbi_construct_lh_part")
        self.n = ctl.nd
        _register(self, 2)

    def matvec(self, u):
        """HACApK_adot_lattice_hyp: au = H u (cluster order, host arrays)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        au = np.zeros(self.n)
        _check(lib().hbi_adot_lattice_hyp(_p(au), self.h, self.ctl.h, None, _p(u)), "hbi_adot_lattice_hyp")
        return au

    def matvec_dev(self, d_au, d_u, stream=0, phase=0):
        """Product on device pointers (ints), enqueued on `stream`; phase 1,
        2 or 3 runs one phase of it alone (for timing), 0 the whole product."""
        _check(lib().hbi_adot_lattice_hyp_phase_dev(C.c_void_p(d_au), self.h, C.c_void_p(d_u), C.c_void_p(stream),
                                                    int(phase)), "hbi_adot_lattice_hyp_phase_dev")

    def tuning(self):
        """The launch shapes the autotuner chose for phases 1 and 2 and the
        median time (us) of every compiled shape per phase."""
        sh1, sh2 = stream_shapes(1), stream_shapes(2)
        s1, s2, src = C.c_int(), C.c_int(), C.c_int()
        us = np.zeros(len(sh1) + len(sh2), dtype=np.float32)
        _check(lib().hbi_lh_tuning(self.h, C.byref(s1), C.byref(s2), us.ctypes.data_as(C.POINTER(C.c_float)),
                                   C.byref(src)), "hbi_lh_tuning")
        def name(t, phase):
            variant = (" col" if t[3] else "") if phase == 1 else (" gather+2" if t[3] else "")
            sched = {0: "", 1: " blocks", 2: " dynamic", 3: " block-shared"}[t[4]]
            return "%dw x %d x %d KB%s%s" % (t[0], t[1], t[2] // 1024, variant, sched)
        return {"phase1": name(sh1[s1.value], 1), "phase2": name(sh2[s2.value], 2), "shape1": s1.value,
                "shape2": s2.value, "source": {0: "timed", 1: "reused", 2: "forced"}.get(src.value, "?"),
                "phase1_us": {name(t, 1): round(float(us[i]), 2) for i, t in enumerate(sh1)},
                "phase2_us": {name(t, 2): round(float(us[len(sh1) + i]), 2) for i, t in enumerate(sh2)}}

    def set_shapes(self, shape1, shape2):
        """Pin the launch shapes (indices into stream_shapes()) of phases 1 and 2."""
        _check(lib().hbi_lh_set_shapes(self.h, int(shape1), int(shape2)), "hbi_lh_set_shapes")

    def check_error(self):
        """hbi_lh_check_error: raises HBIError (code HBI_ERR_DEVICE) if a
        product kernel gave up a bulk-copy wait since the last check; call
        after the stream of matvec_dev products has been synchronised."""
        _check(lib().hbi_lh_check_error(self.h), "hbi_lh_check_error")

    def set_wait_limit(self, cycles):
        """Test hook: bound of the product kernels' bulk-copy waits (SM clock
        cycles; 0 = every wait gives up before its first probe; negative = the
        default).  An ensemble created on the operator afterwards inherits it."""
        _check(lib().hbi_lh_set_wait_limit(self.h, C.c_longlong(int(cycles))), "hbi_lh_set_wait_limit")

    def phase_bytes(self):
        p1, p2 = C.c_double(), C.c_double()
        _check(lib().hbi_lh_phase_bytes(self.h, C.byref(p1), C.byref(p2)), "hbi_lh_phase_bytes")
        return p1.value, p2.value

    def info(self):
        fe, sb, ab = C.c_int64(), C.c_int64(), C.c_double()
        _check(lib().hbi_lh_info(self.h, C.byref(fe), C.byref(sb), C.byref(ab)), "hbi_lh_info")
        return {"factor_elems": fe.value, "store_bytes": sb.value, "alg_bytes": ab.value}

    def close(self):
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_free_lh(self.h)
        self.h = None

    def __del__(self):
        self.close()


# ---- HACApK-named functions (the drop-in surface) -----------------------
def HACApK_init(nd):
    return Ctl(nd)


def HACApK_generate(ctl, geom, ztol):
    return LeafMtxp(ctl, geom, ztol)


def HACApK_construct_LH(lf, ctl, storage=STORE_F64):
    return LHp(lf, ctl, storage)


def HACApK_gen_lattice_vector(ctl):
    ndc = C.c_int()
    lodc = np.zeros(ctl.nd, dtype=np.int32)
    _check(lib().hbi_gen_lattice_vector(ctl.h, C.byref(ndc), lodc.ctypes.data_as(_ip)), "hbi_gen_lattice_vector")
    return ndc.value, lodc


def HACApK_adot_lattice_hyp(lh, u):
    return lh.matvec(u)


def cluster_structure(coord, param=None):
    """Host-only tree + admissibility + leaf order (no GPU).  coord (nd,3)."""
    coord = np.asarray(coord, dtype=np.float64)
    nd = coord.shape[0]
    cf = np.asfortranarray(coord).ravel(order="F")
    lod = np.zeros(nd, dtype=np.int32)
    nl = C.c_int(0)
    pp = _p(np.ascontiguousarray(param, dtype=np.float64)) if param is not None else None
    _check(lib().hbi_cluster_structure(nd, _p(cf), pp, lod.ctypes.data_as(_ip), C.byref(nl), None),
           "hbi_cluster_structure")
    leaves = np.zeros((nl.value, 6), dtype=np.int32)
    _check(lib().hbi_cluster_structure(nd, _p(cf), pp, lod.ctypes.data_as(_ip), C.byref(nl),
                                       leaves.ctypes.data_as(_ip)), "hbi_cluster_structure")
    return lod, leaves


def entry_ij(geom, i, j):
    """HACApK_entry_ij on the GPU for arrays of 1-based (i, j)."""
    i = np.ascontiguousarray(i, dtype=np.int32)
    j = np.ascontiguousarray(j, dtype=np.int32)
    out = np.zeros(len(i))
    _check(lib().hbi_entry_ij(C.byref(geom.bemv), len(i), i.ctypes.data_as(_ip), j.ctypes.data_as(_ip), _p(out)),
           "hbi_entry_ij")
    return out


class RK:
    """derivs / rkck / rkqs of main_LH.f90 on the device (state in cluster order)."""

    def __init__(self, lh_s, lh_n=None, evlaw=0, backslip=1, limitsigma=1, vref=float(np.float32(1e-6)),
                 minsig=1.0, maxsig=300.0, scale=1.0, **params):
        n = lh_s.n
        self.keep = {}
        p = RsfParams()
        p.ncell, p.evlaw, p.backslip, p.limitsigma = n, evlaw, backslip, limitsigma
        p.vref, p.minsig, p.maxsig, p.scale_s, p.scale_n = vref, minsig, maxsig, scale, scale
        for k in ("a", "b", "dc", "f0", "taudot", "sigdot", "vpl"):
            a = np.ascontiguousarray(np.broadcast_to(params.get(k, 0.0), (n,)), dtype=np.float64)
            self.keep[k] = a
            setattr(p, k, _p(a))
        self.h = C.c_void_p()
        _check(lib().hbi_rk_create(C.byref(self.h), C.byref(p), lh_s.h, lh_n.h if lh_n is not None else None),
               "hbi_rk_create")
        self.n, self.lh = n, (lh_s, lh_n)
        self._loops = weakref.WeakSet()  # time loops running on this handle's stream
        _register(self, 1)

    def set_state(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64)
        _check(lib().hbi_rk_set_state(self.h, _p(y)), "hbi_rk_set_state")

    def get_state(self):
        y = np.zeros(3 * self.n)
        _check(lib().hbi_rk_get_state(self.h, _p(y)), "hbi_rk_get_state")
        return y

    def derivs(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64)
        d = np.zeros(3 * self.n)
        _check(lib().hbi_derivs(self.h, _p(y), _p(d)), "hbi_derivs")
        return d

    def rkck(self, h, eps=1.0):
        yo, ye = np.zeros(3 * self.n), np.zeros(3 * self.n)
        em = C.c_double()
        _check(lib().hbi_rkck(self.h, C.c_double(h), C.c_double(eps), _p(yo), _p(ye), C.byref(em)), "hbi_rkck")
        return yo, ye, em.value

    def rkck_into(self, h, eps, yout, yerr):
        """rkck writing into caller-provided (e.g. pinned) float64 arrays."""
        em = C.c_double()
        _check(lib().hbi_rkck(self.h, C.c_double(h), C.c_double(eps), _p(yout), _p(yerr), C.byref(em)), "hbi_rkck")
        return em.value

    def rkqs(self, x, htry, eps, dtmax=1e10):
        xx, hd, hn, em, nr = C.c_double(x), C.c_double(), C.c_double(), C.c_double(), C.c_int()
        _check(lib().hbi_rkqs(self.h, C.byref(xx), C.c_double(htry), C.c_double(eps), C.c_double(dtmax),
                              C.byref(hd), C.byref(hn), C.byref(em), C.byref(nr)), "hbi_rkqs")
        return xx.value, hd.value, hn.value, em.value, nr.value

    @property
    def launches_per_attempt(self):
        return lib().hbi_rk_launches_per_attempt(self.h)

    @property
    def stream(self):
        """cudaStream_t (as int) the handle enqueues on."""
        lib().hbi_rk_stream.restype = C.c_void_p
        return lib().hbi_rk_stream(self.h) or 0

    def check_error(self):
        """Waits for the handle's stream; raises HBIError (HBI_ERR_DEVICE) if a
        product kernel gave up a bulk-copy wait."""
        _check(lib().hbi_rk_check_error(self.h), "hbi_rk_check_error")

    def attempt_async(self, h, eps):
        """Enqueue one Cash-Karp attempt; no host synchronisation."""
        _check(lib().hbi_rk_attempt_async(self.h, C.c_double(h), C.c_double(eps)), "hbi_rk_attempt_async")

    def close(self):
        # a time loop issues its work on this handle's stream: free it first
        # (the garbage collector may finalise the two in either order)
        for c in list(getattr(self, "_loops", ())):
            c.close()
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_rk_free(self.h)
        self.h = None

    def __del__(self):
        self.close()


class Cycle:
    """The time loop of main_LH.f90 (:1217-1438) on the device: rkqs, slip
    update, monitors, events, field output and stop controls.

    Reference defaults (main_LH.f90:133-160): velth=1e-2 and vref=1e-6 are
    default-real literals there, so they are widened from float32 here too.
    """

    def __init__(self, rk, vel, ds, eps_r=1e-4, dtinit=1.0, dtmax=1e10, tmax_yr=1e4,
                 velth=float(np.float32(1e-2)), velmax=1e7, velmin=1e-20, dtout_yr=1.0, dtout_co=1000.0,
                 rigid=32.04, nstep=1000000, interval=0, number=0, outdir=None, inflight=4, restart=False):
        """restart=True continues the run whose files are in outdir (vel is then ignored)."""
        p = CycleParams()
        p.eps_r, p.dtinit, p.dtmax, p.tmax = eps_r, dtinit, dtmax, tmax_yr * YEAR
        p.velth, p.velmax, p.velmin = velth, velmax, velmin
        p.dtout_inter, p.dtout_co, p.rigid = dtout_yr * YEAR, dtout_co, rigid
        p.nstep, p.interval, p.number, p.inflight = nstep, interval, number, inflight
        self._outdir = outdir.encode() if outdir else None
        p.outdir = self._outdir
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        ds = np.ascontiguousarray(ds, dtype=np.float64)
        self.h = C.c_void_p()
        if restart:
            _check(lib().hbi_cycle_restart(C.byref(self.h), rk.h, _p(ds), C.byref(p)), "hbi_cycle_restart")
        else:
            _check(lib().hbi_cycle_create(C.byref(self.h), rk.h, _p(vel), _p(ds), C.byref(p)), "hbi_cycle_create")
        self.rk, self.n = rk, rk.n
        rk._loops.add(self)
        _register(self, 0)

    def run(self, k_limit=0, t_limit=0.0):
        """Run until a stop control, k == k_limit (>0) or x == t_limit (>0, s)."""
        st = CycleStatus()
        _check(lib().hbi_cycle_run(self.h, C.c_longlong(int(k_limit)), C.c_double(t_limit), C.byref(st)),
               "hbi_cycle_run")
        d = st.as_dict()
        d["stop_name"] = STOP_NAMES.get(d["stop"], "?")
        return d

    def fields(self):
        vel, slip = np.zeros(self.n), np.zeros(self.n)
        _check(lib().hbi_cycle_fields(self.h, _p(vel), _p(slip)), "hbi_cycle_fields")
        return vel, slip

    def events(self):
        cnt = C.c_int()
        _check(lib().hbi_cycle_events(self.h, None, 0, C.byref(cnt)), "hbi_cycle_events")
        arr = (Event * max(1, cnt.value))()
        _check(lib().hbi_cycle_events(self.h, arr, cnt.value, C.byref(cnt)), "hbi_cycle_events")
        return [{f: getattr(arr[i], f) for f, _ in Event._fields_} for i in range(cnt.value)]

    def trace(self):
        """Per attempt: k, x, h, errmax, accepted, mvel, hnext, nrjct."""
        cnt = C.c_longlong()
        _check(lib().hbi_cycle_trace(self.h, None, 0, C.byref(cnt)), "hbi_cycle_trace")
        out = np.zeros((cnt.value, 8))
        if cnt.value:
            _check(lib().hbi_cycle_trace(self.h, _p(out), cnt.value, C.byref(cnt)), "hbi_cycle_trace")
        return out

    def set_proposer(self, w):
        """Learned step-size proposer weights (float32 vector), or None to turn it off."""
        if w is None:
            _check(lib().hbi_cycle_set_proposer(self.h, None), "hbi_cycle_set_proposer")
            return
        w = np.ascontiguousarray(w, dtype=np.float32)
        nin, hid, nf = proposer_size()
        if w.size != nf:
            raise ValueError(f"proposer weights: {w.size} floats, expected {nf}")
        _check(lib().hbi_cycle_set_proposer(self.h, w.ctypes.data_as(C.POINTER(C.c_float))), "hbi_cycle_set_proposer")

    def close(self):
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_cycle_free(self.h)
        self.h = None

    def __del__(self):
        self.close()


def proposer_size():
    """(inputs, hidden width, floats in the weight vector) of the step-size proposer."""
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    _check(lib().hbi_cycle_proposer_size(C.byref(a), C.byref(b), C.byref(c)), "hbi_cycle_proposer_size")
    return a.value, b.value, c.value


_fp = C.POINTER(C.c_float)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """nin -> hid -> hid -> 1 MLP trained on the GPU by the library's own
    forward/backward/Adam kernels (hbi_mlp_*)."""

    def __init__(self, nin, hid, batch_max=4096):
        self.nin, self.hid = nin, hid
        self.np = hid * nin + hid + hid * hid + hid + hid + 1
        self.h = C.c_void_p()
        _check(lib().hbi_mlp_create(C.byref(self.h), nin, hid, batch_max), "hbi_mlp_create")
        _register(self, 0)

    def init(self, seed=0):
        """Glorot-uniform weights, zero biases."""
        rng = np.random.default_rng(seed)
        p = np.zeros(self.np, dtype=np.float32)
        nin, h = self.nin, self.hid
        o = 0
        for fan_in, fan_out in ((nin, h), (h, h), (h, 1)):
            lim = np.sqrt(6.0 / (fan_in + fan_out))
            p[o:o + fan_in * fan_out] = rng.uniform(-lim, lim, fan_in * fan_out)
            o += fan_in * fan_out + fan_out
        self.set_params(p)
        return p

    def set_loss(self, tau=None):
        """Squared error (tau None), or the pinball loss of quantile tau."""
        _check(lib().hbi_mlp_set_loss(self.h, C.c_float(-1.0 if tau is None else tau)), "hbi_mlp_set_loss")

    def set_params(self, p):
        p = _f32(p)
        _check(lib().hbi_mlp_set_params(self.h, p.ctypes.data_as(_fp)), "hbi_mlp_set_params")

    def params(self):
        p = np.zeros(self.np, dtype=np.float32)
        _check(lib().hbi_mlp_get_params(self.h, p.ctypes.data_as(_fp)), "hbi_mlp_get_params")
        return p

    def loss_grad(self, x, t):
        x, t = _f32(x), _f32(t)
        g = np.zeros(self.np, dtype=np.float32)
        out = np.zeros(len(t), dtype=np.float32)
        loss = C.c_float()
        _check(lib().hbi_mlp_loss_grad(self.h, x.ctypes.data_as(_fp), t.ctypes.data_as(_fp), len(t),
                                       g.ctypes.data_as(_fp), C.byref(loss), out.ctypes.data_as(_fp)),
               "hbi_mlp_loss_grad")
        return float(loss.value), g, out

    def train(self, x, t, epochs=50, batch=1024, lr=1e-3, seed=0):
        x, t = _f32(x), _f32(t)
        hist = np.zeros(epochs, dtype=np.float32)
        _check(lib().hbi_mlp_train(self.h, x.ctypes.data_as(_fp), t.ctypes.data_as(_fp), C.c_longlong(len(t)),
                                   epochs, batch, C.c_float(lr), C.c_ulonglong(seed), hist.ctypes.data_as(_fp)),
               "hbi_mlp_train")
        return hist

    def predict(self, x):
        x = _f32(x)
        out = np.zeros(len(x), dtype=np.float32)
        _check(lib().hbi_mlp_predict(self.h, x.ctypes.data_as(_fp), C.c_longlong(len(x)), out.ctypes.data_as(_fp)),
               "hbi_mlp_predict")
        return out

    def close(self):
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_mlp_free(self.h)
        self.h = None

    def __del__(self):
        self.close()


def stream_shapes(phase=1):
    """The compiled launch shapes of the phase-1 or phase-2 product kernel:
    [(warps per block, stages per warp, stage bytes, variant, schedule), ...]."""
    k = C.c_int()
    _check(lib().hbi_stream_shapes(int(phase), C.byref(k), None), "hbi_stream_shapes")
    a = np.zeros(5 * k.value, dtype=np.int32)
    _check(lib().hbi_stream_shapes(int(phase), C.byref(k), a.ctypes.data_as(_ip)), "hbi_stream_shapes")
    return [tuple(int(v) for v in a[5 * s:5 * s + 5]) for s in range(k.value)]


def plan_block_schedule(cost, key, nblocks, nw):
    """The block schedule with locality (hbi_plan_block_schedule): returns
    (woff[nblocks * nw + 1], witem[n])."""
    cost = np.ascontiguousarray(cost, dtype=np.int64)
    key = np.ascontiguousarray(key, dtype=np.int64)
    woff = np.zeros(nblocks * nw + 1, dtype=np.int32)
    witem = np.zeros(max(len(cost), 1), dtype=np.int32)
    _check(lib().hbi_plan_block_schedule(len(cost), cost.ctypes.data_as(_i64p), key.ctypes.data_as(_i64p),
                                         int(nblocks), int(nw), woff.ctypes.data_as(_ip), witem.ctypes.data_as(_ip)),
           "hbi_plan_block_schedule")
    return woff, witem[:len(cost)]


def autotune_select(times):
    """The autotuner's selection rule (host only): times (candidates x
    repeats) -> (best candidate, medians)."""
    t = np.ascontiguousarray(times, dtype=np.float32)
    med = np.zeros(t.shape[0], dtype=np.float32)
    best = C.c_int()
    _check(lib().hbi_autotune_select(t.shape[0], t.shape[1], t.ctypes.data_as(C.POINTER(C.c_float)),
                                     med.ctypes.data_as(C.POINTER(C.c_float)), C.byref(best)), "hbi_autotune_select")
    return best.value, med


def partition_leaves(leaves, nranks):
    """Deal the leaves (nleaf x 6 table) to nranks ranks by factor elements
    (host only): returns (owner per leaf, elements per rank)."""
    lv = np.ascontiguousarray(leaves, dtype=np.int32)
    owner = np.zeros(max(len(lv), 1), dtype=np.int32)
    load = np.zeros(nranks, dtype=np.int64)
    _check(lib().hbi_partition_leaves(len(lv), lv.ctypes.data_as(_ip), int(nranks), owner.ctypes.data_as(_ip),
                                      load.ctypes.data_as(_i64p)), "hbi_partition_leaves")
    return owner[:len(lv)], load


def plan_warp_schedule(cost, nwarps):
    """The product kernels' static warp schedule (hbi_plan_warp_schedule):
    returns (woff[nwarps + 1], witem[n])."""
    cost = np.ascontiguousarray(cost, dtype=np.int64)
    woff = np.zeros(nwarps + 1, dtype=np.int32)
    witem = np.zeros(max(len(cost), 1), dtype=np.int32)
    _check(lib().hbi_plan_warp_schedule(len(cost), cost.ctypes.data_as(_i64p), int(nwarps),
                                        woff.ctypes.data_as(_ip), witem.ctypes.data_as(_ip)),
           "hbi_plan_warp_schedule")
    return woff, witem[:len(cost)]


def plan_emulate(n, leaves, body, vec, x):
    """Host walk of the product's work plan (hbi_plan_emulate): y = H x and
    plan statistics, without a GPU.  leaves: (nleaf, 6) int array
    {ltmtx, kt, nstrtl, ndl, nstrtt, ndt}; body: HACApK-packed FP64 factors."""
    lv = np.ascontiguousarray(leaves, dtype=np.int32)
    body = np.ascontiguousarray(body, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(n)
    st = np.zeros(8, dtype=np.int64)
    _check(lib().hbi_plan_emulate(n, len(lv), lv.ctypes.data_as(_ip), _p(body), vec, _p(x), _p(y),
                                  st.ctypes.data_as(_i64p)), "hbi_plan_emulate")
    keys = ("items1", "items2", "vstore", "ustore", "zlen", "plen1", "plen2", "segments")
    return y, dict(zip(keys, (int(v) for v in st)))


def umma_probe(a_bf16_bits, b_bf16_bits, variant=0):
    """One tcgen05 MMA on the GPU: (128x16) x (64x16)^T from BF16 bit patterns."""
    a = np.ascontiguousarray(a_bf16_bits, dtype=np.uint16)
    b = np.ascontiguousarray(b_bf16_bits, dtype=np.uint16)
    d = np.zeros((128, 64), dtype=np.float32)
    _check(lib().hbi_umma_probe(a.ctypes.data_as(C.POINTER(C.c_uint16)), b.ctypes.data_as(C.POINTER(C.c_uint16)),
                                d.ctypes.data_as(_fp), int(variant)), "hbi_umma_probe")
    return d


class EnsStatus(C.Structure):
    _fields_ = [("attempts", C.c_longlong), ("steps", C.c_longlong), ("rejected", C.c_longlong),
                ("done", C.c_int), ("failed", C.c_int), ("wall_s", C.c_double)]


class Ensemble:
    """64 rate-and-state systems with their own b and dc sharing one pair of
    FP32 H-matrices (hbi_ens_*): one multi-vector product per stage, FP64
    per-member state and rkqs controllers.  b, dc: (n, 64) arrays in cluster
    order; other parameters as RK."""

    MEMBERS = 64

    def __init__(self, lh_s, lh_n, b, dc, evlaw=0, backslip=1, limitsigma=1, vref=float(np.float32(1e-6)),
                 minsig=1.0, maxsig=300.0, scale=1.0, **params):
        n = lh_s.n
        self.keep = {}
        p = RsfParams()
        p.ncell, p.evlaw, p.backslip, p.limitsigma = n, evlaw, backslip, limitsigma
        p.vref, p.minsig, p.maxsig, p.scale_s, p.scale_n = vref, minsig, maxsig, scale, scale
        for k in ("a", "f0", "taudot", "sigdot", "vpl"):
            a = np.ascontiguousarray(np.broadcast_to(params.get(k, 0.0), (n,)), dtype=np.float64)
            self.keep[k] = a
            setattr(p, k, _p(a))
        zero = np.zeros(n)
        self.keep["z"] = zero
        p.b, p.dc = _p(zero), _p(zero)
        b = np.ascontiguousarray(np.broadcast_to(b, (n, self.MEMBERS)), dtype=np.float64)
        dc = np.ascontiguousarray(np.broadcast_to(dc, (n, self.MEMBERS)), dtype=np.float64)
        self.h = C.c_void_p()
        _check(lib().hbi_ens_create(C.byref(self.h), C.byref(p), lh_s.h, lh_n.h if lh_n is not None else None,
                                    self.MEMBERS, _p(b), _p(dc)), "hbi_ens_create")
        self.n, self.lh = n, (lh_s, lh_n)
        _register(self, 1)

    def set_state(self, y, vel):
        """y: (3n, 64) [psi, tau, sigma per element], vel: (n, 64)."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        _check(lib().hbi_ens_set_state(self.h, _p(y), _p(vel)), "hbi_ens_set_state")

    def get_state(self):
        y = np.zeros((3 * self.n, self.MEMBERS))
        slip = np.zeros((self.n, self.MEMBERS))
        x = np.zeros(self.MEMBERS)
        _check(lib().hbi_ens_get_state(self.h, _p(y), _p(slip), _p(x)), "hbi_ens_get_state")
        return y, slip, x

    def use_tensor_cores(self, lf_s, lf_n=None):
        """Switch the multi-vector product to the tcgen05 kernels (FP64
        factors of the LeafMtxp handles, stored as BF16 hi + lo)."""
        _check(lib().hbi_ens_use_tensor_cores(self.h, lf_s.h, lf_n.h if lf_n is not None else None),
               "hbi_ens_use_tensor_cores")
        self.lf = (lf_s, lf_n)

    def product(self, x, reps=0):
        """One multi-vector product of both H-matrices on the 64 members'
        vectors x (n, 64), cluster order (hbi_ens_product): returns (ys, yn,
        ms per product or None)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.shape != (self.n, 64):
            raise ValueError(f"x: shape {x.shape}, expected ({self.n}, 64)")
        ys, yn = np.zeros_like(x), np.zeros_like(x)
        ms = C.c_double(0.0)
        _check(lib().hbi_ens_product(self.h, x.ctypes.data_as(_fp), ys.ctypes.data_as(_fp),
                                     yn.ctypes.data_as(_fp), int(reps), C.byref(ms)), "hbi_ens_product")
        return ys, yn, (ms.value if reps > 0 else None)

    def run(self, t_limit, eps_r=1e-6, dtinit=1.0, dtmax=1e10):
        st = EnsStatus()
        _check(lib().hbi_ens_run(self.h, C.c_double(eps_r), C.c_double(dtinit), C.c_double(dtmax),
                                 C.c_double(t_limit), C.byref(st)), "hbi_ens_run")
        return {f: getattr(st, f) for f, _ in EnsStatus._fields_}

    def close(self):
        if getattr(self, "h", None) and _lib is not None and not _closed:
            _lib.hbi_ens_free(self.h)
        self.h = None

    def __del__(self):
        self.close()


def tc_plan_emulate(n, leaves, body, x):
    """Host walk of the ensemble's tensor-core plan (hbi_tc_plan_emulate)."""
    lv = np.ascontiguousarray(leaves, dtype=np.int32)
    body = np.ascontiguousarray(body, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(n)
    st = np.zeros(4, dtype=np.int64)
    _check(lib().hbi_tc_plan_emulate(n, len(lv), lv.ctypes.data_as(_ip), _p(body), _p(x), _p(y),
                                     st.ctypes.data_as(_i64p)), "hbi_tc_plan_emulate")
    return y, dict(zip(("items1", "items2", "store1", "store2"), (int(v) for v in st)))


def restart_point(monitor_path, interval):
    """(k, x, next trial step, last step listed) of a monitor file (host only)."""
    k, kend = C.c_longlong(), C.c_longlong()
    x, dt = C.c_double(), C.c_double()
    _check(lib().hbi_restart_point(str(monitor_path).encode(), C.c_longlong(interval), C.byref(k), C.byref(x),
                                   C.byref(dt), C.byref(kend)), "hbi_restart_point")
    return k.value, x.value, dt.value, kend.value
