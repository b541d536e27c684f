"""Seeded synthetic workloads with the shapes of the five benchmark
configurations, and the driver-side setup of main_LH.f90 around the hot path
(parameters mapped to cluster order through lodc, initial state psi from
steady state, loading by back slip).

The SEAS benchmark data and the reference's missing example files are not
available; every field here is generated from a seed.
"""
import math

import numpy as np

from . import HBI_2DVS, HBI_3DPH, HBI_3DNR, HBI_3DNT, Geometry
from . import mesh

RIGID, VS = 32.04, 3.464
VREF = float(np.float32(1e-6))  # main_LH.f90:134 default vref=1e-6 (default-real literal)


class Workload:
    """Geometry + per-element friction parameters (global order)."""

    def __init__(self, name, problem, nd, geom_kw, nmat, evlaw, ds_area, params, eps_h, tmax_yr, scale=1.0,
                 w=0.0, lb_ds=None):
        self.name, self.problem, self.nd = name, problem, nd
        self.geom_kw, self.nmat, self.evlaw = geom_kw, nmat, evlaw
        self.ds_area = ds_area
        self.params = params  # global order: a b dc f0 sigma vel vpl taudot sigdot
        self.eps_h, self.tmax_yr, self.scale, self.w = eps_h, tmax_yr, scale, w

    def geometry(self, v="s"):
        return Geometry(self.problem, self.nd, v=v, w=self.w, **self.geom_kw)

    def initial_state(self, lodc):
        """psi, tau, sigma in cluster order (main_LH.f90:973-1004)."""
        idx = lodc - 1
        p = {k: v[idx] for k, v in self.params.items()}
        a, b, f0, sig, vel = p["a"], p["b"], p["f0"], p["sigma"], p["vel"]
        # shear stress at steady state for the initial slip rate
        psi_ss = f0 - b * np.log(vel / VREF)
        tau = a * sig * np.arcsinh(vel / (2 * VREF) * np.exp(psi_ss / a))
        psi = a * np.log(2 * VREF / vel * np.sinh(tau / sig / a))
        y = np.empty(3 * self.nd)
        y[0::3], y[1::3], y[2::3] = psi, tau, sig
        return y, p


def c1_2dvs(n=1024, seed=0):
    """2D antiplane strike slip, 40 km deep, aging law, b tapering below 15 km."""
    ds0 = 40.0 / n
    xel, xer, xcol, ds = mesh.mesh_2dp(n, ds0)
    b = np.where(xcol <= 15.0, 0.015, np.where(xcol <= 18.0, 0.015 - (0.010) * (xcol - 15.0) / 3.0, 0.005))
    rng = np.random.default_rng(seed)
    vel = 1e-9 * (1.0 + 0.01 * rng.uniform(-1, 1, n))
    params = dict(a=np.full(n, 0.010), b=b, dc=np.full(n, 0.008), f0=np.full(n, 0.6), sigma=np.full(n, 50.0),
                  vel=vel, vpl=np.full(n, 1e-9), taudot=np.zeros(n), sigdot=np.zeros(n))
    return Workload("c1_2dvs_1024", HBI_2DVS, n, dict(xcol=xcol, xel=xel, xer=xer), 1, 0, ds, params, 1e-6, 1500.0)


def c2_3dph(imax=256, jmax=256, ds0=0.2, seed=0, b_in=0.014, dc=0.02):
    """30-degree thrust, Okada half space, velocity-weakening central patch."""
    xcol, ycol, zcol, angd, ang = mesh.mesh_3ddip(imax, jmax, ds0, 30.0)
    n = imax * jmax
    rake = np.full(n, 90.0 / 180.0 * mesh.PI)
    # down-dip distance of each element
    ii = np.repeat(np.arange(imax), jmax)
    jj = np.tile(np.arange(jmax), imax)
    inside = (np.abs(ii - imax / 2 + 0.5) < 0.35 * imax) & (np.abs(jj - jmax / 2 + 0.5) < 0.35 * jmax)
    a = np.full(n, 0.010)
    b = np.where(inside, np.broadcast_to(b_in, (n,)), 0.006) if np.ndim(b_in) == 0 else np.where(inside, b_in, 0.006)
    dcv = np.broadcast_to(np.asarray(dc, dtype=np.float64), (n,)).copy()
    # V = vpl everywhere is a fixed point of the back-slip-loaded system (the
    # error estimate is zero and rkqs cannot step); seeded 1% noise as in c1
    vel = 1e-9 * (1.0 + 0.01 * np.random.default_rng(seed).uniform(-1, 1, n))
    params = dict(a=a, b=b, dc=dcv, f0=np.full(n, 0.6), sigma=np.full(n, 50.0), vel=vel,
                  vpl=np.full(n, 1e-9), taudot=np.zeros(n), sigdot=np.zeros(n))
    g = dict(xcol=xcol, ycol=ycol, zcol=zcol, ang=ang, angd=angd, dsl=np.full(n, ds0), dsd=np.full(n, ds0),
             rake=rake)
    return Workload(f"c2_3dph_{imax}x{jmax}", HBI_3DPH, n, g, 2, 0, np.full(n, ds0 * ds0), params, 1e-5, 500.0,
                    scale=1.0 / ds0, w=ds0)


def c3_3dnt(nx=500, nz=200, length=60.0, width=30.0, seed=0, eps_h=1e-4):
    """Rough strike-slip fault on triangles, TDstressFS full space, slip law."""
    tri = mesh.rough_fault(nx, nz, length, width, seed=seed)
    g, area = mesh.tri_geometry(tri)
    n = tri.shape[0]
    rng = np.random.default_rng(seed + 1)
    ln = lambda m: m * np.exp(0.1 * rng.standard_normal(n))
    a, b, dc = ln(0.01), ln(0.014), ln(0.01)
    vel = 1e-9 * (1.0 + 0.01 * rng.uniform(-1, 1, n))
    params = dict(a=a, b=b, dc=dc, f0=np.full(n, 0.6), sigma=np.full(n, 50.0),
                  vel=vel, vpl=np.full(n, 1e-9), taudot=np.zeros(n), sigdot=np.zeros(n))
    g["rake"] = np.zeros(n)
    return Workload(f"c3_3dnt_{n}", HBI_3DNT, n, g, 2, 1, area, params, eps_h, 100.0)


def c5_3dnt(seed=0):
    """Configuration 5: the c3 fault meshed with 500,000 triangles."""
    w = c3_3dnt(1000, 250, seed=seed)
    w.name = f"c5_3dnt_{w.nd}"
    return w


def ensemble_params(M=64, seed=0):
    """c4: per-member b in [0.012, 0.018] and Dc in [5, 30] mm."""
    rng = np.random.default_rng(seed)
    return rng.uniform(0.012, 0.018, M), rng.uniform(0.005, 0.030, M)


def ensemble_state(w, lodc, b_in, dc_m):
    """c4 on a c2 workload: per-member b (b_in inside the velocity-weakening
    patch, the workload's b outside) and dc, and each member's steady initial
    state; arrays (n, M) / (3n, M) in cluster order, member index fastest."""
    idx = lodc - 1
    p = {k: v[idx] for k, v in w.params.items()}
    M = len(b_in)
    inside = p["b"] > 0.01  # the patch carries b_in, the frame 0.006
    b = np.where(inside[:, None], np.asarray(b_in)[None, :], p["b"][:, None])
    dc = np.broadcast_to(np.asarray(dc_m)[None, :], (w.nd, M)).copy()
    a, f0, sig, vel = p["a"][:, None], p["f0"][:, None], p["sigma"][:, None], p["vel"][:, None]
    psi_ss = f0 - b * np.log(vel / VREF)
    tau = a * sig * np.arcsinh(vel / (2 * VREF) * np.exp(psi_ss / a))
    psi = a * np.log(2 * VREF / vel * np.sinh(tau / sig / a))
    y = np.empty((3 * w.nd, M))
    y[0::3], y[1::3], y[2::3] = psi, tau, np.broadcast_to(sig, (w.nd, M))
    return y, np.broadcast_to(vel, (w.nd, M)).copy(), b, dc, p
