"""Small seeded workloads shared by the GPU parity tests and smoke()."""
import numpy as np

import hbi_gb300 as H
from hbi_gb300 import mesh


def case(kind, n_hint=None):
    """Returns (problem, nd, geometry kwargs, w, eps_h)."""
    if kind == "2dvs":
        n = n_hint or 512
        xel, xer, xcol, _ = mesh.mesh_2dp(n, 40.0 / n)
        return H.HBI_2DVS, n, dict(xcol=xcol, xel=xel, xer=xer), 0.0, 1e-6
    if kind in ("3dph", "3dnr"):
        imax, jmax = (n_hint or (32, 16))
        ds0 = 0.2
        xcol, ycol, zcol, angd, ang = mesh.mesh_3ddip(imax, jmax, ds0, 30.0)
        n = imax * jmax
        g = dict(xcol=xcol, ycol=ycol, zcol=zcol, ang=ang, angd=angd, dsl=np.full(n, ds0), dsd=np.full(n, ds0),
                 rake=np.full(n, 90.0 / 180.0 * mesh.PI))
        return (H.HBI_3DPH if kind == "3dph" else H.HBI_3DNR), n, g, ds0, 1e-5
    if kind == "3dnt":
        nx, nz = (n_hint or (24, 12))
        tri = mesh.rough_fault(nx, nz, 6.0, 3.0, seed=5)
        g, _ = mesh.tri_geometry(tri)
        n = len(tri)
        g["rake"] = np.zeros(n)
        return H.HBI_3DNT, n, g, 0.0, 1e-4
    if kind == "3dht":
        nx, nz = (n_hint or (24, 12))
        tri = mesh.rough_fault(nx, nz, 6.0, 3.0, seed=7)
        tri[:, :, 2] -= 0.5  # buried: top edge 0.5 km below the free surface
        g, _ = mesh.tri_geometry(tri)
        n = len(tri)
        g["rake"] = np.linspace(0.0, 0.5 * mesh.PI, n)  # the source's own rake enters the 3dht entry
        return H.HBI_3DHT, n, g, 0.0, 1e-4
    if kind == "2dph":
        n = n_hint or 600
        xel, xer, yel, yer, xcol, ycol, ang, _ = mesh.mesh_2dph(n, 40.0 / n, 30.0)
        return H.HBI_2DPH, n, dict(xcol=xcol, ycol=ycol, zcol=np.zeros(n), xel=xel, xer=xer, yel=yel, yer=yer,
                                   ang=ang), 0.0, 1e-6
    if kind == "2dn":
        n = n_hint or 600
        xel, xer, yel, yer, xcol, ycol, ang, _ = mesh.mesh_2dn(*mesh.bent_fault_2d(n, 40.0, 0.0, 25.0, seed=3,
                                                                                   rough=0.2))
        return H.HBI_2DN, n, dict(xcol=xcol, ycol=ycol, zcol=np.zeros(n), xel=xel, xer=xer, yel=yel, yer=yer,
                                  ang=ang), 0.0, 1e-6
    raise ValueError(kind)


ORC_PROBLEM = {H.HBI_2DVS: 1, H.HBI_3DPH: 2, H.HBI_3DNR: 3, H.HBI_3DNT: 4, H.HBI_2DPH: 5, H.HBI_2DN: 6,
               H.HBI_3DHT: 7}


def oracle_geometry(O, problem, n, g, w, v):
    return O.Geometry(ORC_PROBLEM[problem], n, v, w=w, **g)


def product_geometry(problem, n, g, w, v):
    return H.Geometry(problem, n, v=v, w=w, **g)
