"""Bit-exact cluster tree, admissibility and leaf order: the product's host
builder (hbi_cluster_structure in libhbigpu.so, no GPU needed) against the
oracle restatement of HACApK (m_HACApK_base.f90:2372-2460, 2937-2995,
3114-3166, 3191-3333)."""
import math

import numpy as np
import pytest

import hbi_gb300 as H
from hbi_gb300 import mesh


def _both(oracle, coord, param=None):
    lod_o, lv_o, cnt = oracle.build_structure(coord, param)
    lod_p, lv_p = H.cluster_structure(coord, param)
    return lod_o, lv_o, cnt, lod_p, lv_p


def _check(oracle, coord, param=None):
    lod_o, lv_o, cnt, lod_p, lv_p = _both(oracle, coord, param)
    assert np.array_equal(lod_o, lod_p)
    assert np.array_equal(lv_o[:, [0, 2, 3, 4, 5]], lv_p[:, [0, 2, 3, 4, 5]])
    assert cnt == len(lv_o)
    n = len(coord)
    # the leaves tile the matrix exactly once
    area = (lv_p[:, 3].astype(np.int64) * lv_p[:, 5]).sum()
    assert area == n * n
    assert sorted(lod_p) == list(range(1, n + 1))
    return lv_p


@pytest.mark.parametrize("n", [1, 15, 16, 17, 100, 1024, 1600])
def test_2dvs_structure(oracle, n):
    xel, xer, xcol, _ = mesh.mesh_2dp(n, 40.0 / n)
    _check(oracle, np.stack([xcol, np.zeros(n), np.zeros(n)], 1))


@pytest.mark.parametrize("imax,jmax", [(16, 16), (64, 32), (150, 30)])
def test_3dph_structure(oracle, imax, jmax):
    xcol, ycol, zcol, angd, ang = mesh.mesh_3ddip(imax, jmax, 0.1, 30.0)
    _check(oracle, np.stack([xcol, ycol, zcol], 1))


def test_rough_triangle_structure(oracle):
    tri = mesh.rough_fault(40, 20, 6.0, 3.0, seed=3)
    g, _ = mesh.tri_geometry(tri)
    _check(oracle, np.stack([g["xcol"], g["ycol"], g["zcol"]], 1))


def test_degenerate_points(oracle):
    """Coincident points and ties on the cut plane follow the reference loop."""
    rng = np.random.default_rng(1)
    c = np.round(rng.uniform(0, 4, (500, 3)))  # many exact ties
    _check(oracle, c)
    _check(oracle, np.zeros((40, 3)))


def test_params_change_leaves(oracle):
    xel, xer, xcol, _ = mesh.mesh_2dp(512, 0.1)
    c = np.stack([xcol, np.zeros(512), np.zeros(512)], 1)
    p = oracle.default_params()
    p[20] = 7        # leaf size param(21)
    p[50] = 1.0      # eta param(51)
    lv = _check(oracle, c, p)
    lv0 = _check(oracle, c)
    assert len(lv) != len(lv0)


def test_mesh_builders_match_oracle(oracle):
    a = mesh.mesh_2dp(1000, 0.04)
    b = oracle.mesh_2dp(1000, 0.04)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    a = mesh.mesh_3ddip(20, 12, 0.2, 30.0)
    b = oracle.mesh_3ddip(20, 12, 0.2, 30.0)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    tri = mesh.rough_fault(10, 6, 3.0, 2.0, seed=0)
    xs = [tri[:, k, 0] for k in range(3)] + [tri[:, k, 1] for k in range(3)] + [tri[:, k, 2] for k in range(3)]
    ev_p = mesh.evcalc(*xs)
    ev_o = oracle.evcalc(*xs)
    for x, y in zip(ev_p, ev_o):
        assert np.array_equal(x, y)


def test_stl_roundtrip(tmp_path):
    tri = mesh.rough_fault(5, 4, 2.0, 1.0, seed=2)
    p = tmp_path / "f.stl"
    mesh.write_stl(str(p), tri)
    xs, ys, zs = mesh.read_stl(str(p))
    assert xs.shape == (3, len(tri))
    assert np.array_equal(xs[0], tri[:, 0, 0]) and np.array_equal(zs[2], tri[:, 2, 2])
    # the reference counts facets as lines/7
    assert len(open(p).read().splitlines()) // 7 == len(tri)


def _fort_e(v, w=16, d=5):
    if v == 0:
        s = "0." + "0" * d + "E+00"
    else:
        m, e = f"{abs(v):.{d - 1}e}".split("e")
        e = int(e) + 1
        digits = m.replace(".", "")
        ex = f"E{'+' if e >= 0 else '-'}{abs(e):02d}" if abs(e) <= 99 else f"{'+' if e >= 0 else '-'}{abs(e):03d}"
        s = ("-" if v < 0 else "") + "0." + digits + ex
    return s.rjust(w)


def test_restart_point_follows_the_reference_rule(tmp_path):
    """main_LH.f90:836-849: the last monitor line with k % interval == 0 gives
    x and the next trial step min(2 dtdid, 0.9 dtdid errmax**-0.2); Fortran's
    exponent without its letter (three digits) is read too."""
    lines = []
    for k in range(0, 251):
        x = 1000.0 * k
        errmax, dtdid = 0.25 + 0.001 * k, 10.0 + k
        wall = 1e-120 if k == 200 else 0.5
        l = f"{k:7d}{x:19.4f}" + "".join(_fort_e(v) for v in (-9.0, 1e-3, 0.6, 50.0, 50.0, errmax, dtdid))
        l += f"{0:4d}{wall:16.4f}" if k != 200 else f"{0:4d}" + _fort_e(wall)
        lines.append(l)
    p = tmp_path / "monitor1.dat"
    p.write_text("\n".join(lines) + "\n")
    k, x, dt, kend = H.restart_point(p, 100)
    assert (k, kend) == (200, 250)
    assert x == 200000.0
    e, h = float(_fort_e(0.45)), float(_fort_e(210.0))
    assert abs(dt - min(2 * h, float(np.float32(0.9)) * h * e ** float(np.float32(-0.2)))) <= 1e-12 * dt


def test_2d_meshes_follow_the_reference_builders():
    """coordinate2dph (main_LH.f90:1720-1737): element i from (i-1) ds0 to
    i ds0 along the dip; coordinate2dn (:1739-1750): lengths, angles and
    midpoints of given element ends."""
    n, ds0, dip = 5, 0.25, 30.0
    xel, xer, yel, yer, xcol, ycol, ang, ds = mesh.mesh_2dph(n, ds0, dip)
    c, s = math.cos(dip * mesh.PI / 180), math.sin(dip * mesh.PI / 180)
    for i in range(1, n + 1):
        assert xel[i - 1] == (i - 1) * ds0 * c and xer[i - 1] == i * ds0 * c
        assert yel[i - 1] == (i - 1) * ds0 * s and yer[i - 1] == i * ds0 * s
        assert xcol[i - 1] == 0.5 * (xel[i - 1] + xer[i - 1]) and ycol[i - 1] == 0.5 * (yel[i - 1] + yer[i - 1])
        assert ang[i - 1] == math.atan2(yer[i - 1] - yel[i - 1], xer[i - 1] - xel[i - 1])
    assert np.all(ds == ds0)
    ends = mesh.bent_fault_2d(64, 10.0, 1.0, 30.0, seed=4, rough=0.2)
    assert all(np.array_equal(a, b) for a, b in zip(ends, mesh.bent_fault_2d(64, 10.0, 1.0, 30.0, seed=4, rough=0.2)))
    xel, xer, yel, yer, xcol, ycol, ang, ds = mesh.mesh_2dn(*ends)
    assert np.allclose(ds, 10.0 / 64, rtol=1e-12)
    assert np.array_equal(xel[1:], xer[:-1]) and np.array_equal(yel[1:], yer[:-1])  # a connected trace
