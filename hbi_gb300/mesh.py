"""Fault meshes of the HBI driver (main_LH.f90) and the seeded synthetic
geometries used for the benchmark configurations.

coordinate2dp    main_LH.f90:1701-1718   (2dvs)
coordinate2dph   main_LH.f90:1720-1737   (2dph)
coordinate2dn    main_LH.f90:1739-1750   (2dn / 2dnh, element ends from a geometry file)
coordinate3ddip  main_LH.f90:1781-1835   (3dph)
.stl reader      main_LH.f90:357-368, 485-509 (3dnt; 7 lines per facet)
evcalc           main_LH.f90:1940-1990

Per-element trigonometry uses the `math` module (the C library), so these
arrays are bit-identical to what the reference's compiled code produces with
the same libm; elementwise arithmetic is plain IEEE (numpy applies one
operation at a time, no fused multiply-add).
"""
import math

import numpy as np

PI = 4 * math.atan(1.0)


def mesh_2dp(n, ds0):
    """xel, xer, xcol, ds of a vertical 2D fault of n elements of size ds0."""
    i = np.arange(1, n + 1, dtype=np.float64)
    xel = (i - 1) * ds0
    xer = i * ds0
    xcol = 0.5 * (xel + xer)
    return xel, xer, xcol, np.full(n, float(ds0))


def mesh_2dph(n, ds0, dipangle):
    """xel, xer, yel, yer, xcol, ycol, ang, ds of a planar 2D fault of n
    elements of size ds0 dipping `dipangle` degrees from the free surface
    (y is depth, positive down)."""
    c = math.cos(dipangle * PI / 180)
    s = math.sin(dipangle * PI / 180)
    i = np.arange(1, n + 1, dtype=np.float64)
    xel, xer = (i - 1) * ds0 * c, i * ds0 * c
    yel, yer = (i - 1) * ds0 * s, i * ds0 * s
    return _mesh_2d_from_ends(xel, xer, yel, yer, np.full(n, float(ds0)))


def mesh_2dn(xel, xer, yel, yer):
    """xel, xer, yel, yer, xcol, ycol, ang, ds of a 2D fault given by its
    element ends (the rows of a 2dn / 2dnh geometry file)."""
    xel, xer, yel, yer = (np.asarray(a, dtype=np.float64) for a in (xel, xer, yel, yer))
    ds = np.sqrt((xer - xel) ** 2 + (yer - yel) ** 2)
    return _mesh_2d_from_ends(xel, xer, yel, yer, ds)


def _mesh_2d_from_ends(xel, xer, yel, yer, ds):
    xcol = 0.5 * (xel + xer)
    ycol = 0.5 * (yel + yer)
    ang = np.array([math.atan2(yer[k] - yel[k], xer[k] - xel[k]) for k in range(len(xel))])
    return xel, xer, yel, yer, xcol, ycol, ang, ds


def bent_fault_2d(n, length, depth0, bend_deg, seed=0, rough=0.0):
    """Element ends of a seeded 2D fault for the 2dn / 2dnh problems: a trace
    from depth depth0 whose strike angle turns linearly by bend_deg over its
    length, with optional seeded roughness of relative amplitude `rough`."""
    rng = np.random.default_rng(seed)
    ds = length / n
    turn = np.deg2rad(bend_deg) * np.arange(n) / max(1, n - 1)
    if rough > 0:
        turn = turn + rough * np.cumsum(rng.standard_normal(n)) / math.sqrt(n)
    x = np.concatenate([[0.0], np.cumsum(ds * np.cos(turn))])
    y = depth0 + np.concatenate([[0.0], np.cumsum(ds * np.sin(turn))])
    return x[:-1], x[1:], y[:-1], y[1:]


def mesh_3ddip(imax, jmax, ds0, dipangle):
    """xcol, ycol, zcol, angd, ang of a planar fault dipping `dipangle` degrees."""
    cdip = ds0 * math.cos(dipangle * PI / 180.0)
    sdip = ds0 * math.sin(dipangle * PI / 180.0)
    yr = np.zeros(jmax + 1)
    zr = np.zeros(jmax + 1)
    for j in range(1, jmax + 1):
        yr[j] = yr[j - 1] - cdip
        zr[j] = zr[j - 1] - sdip
    angd_j = np.array([math.atan2(zr[j - 1] - zr[j], yr[j - 1] - yr[j]) for j in range(1, jmax + 1)])
    ii = np.repeat(np.arange(1, imax + 1), jmax)
    xcol = (ii - imax // 2 - 0.5) * ds0
    ycol = np.tile(0.5 * (yr[:-1] + yr[1:]), imax)
    zcol = np.tile(0.5 * (zr[:-1] + zr[1:]), imax)
    angd = np.tile(angd_j, imax)
    return xcol, ycol, zcol, angd, np.zeros(imax * jmax)


def evcalc(xs1, xs2, xs3, ys1, ys2, ys3, zs1, zs2, zs3):
    """Unit normal (ev3*), strike (ev1*) and dip (ev2*) vectors and areas."""
    vba = [xs2 - xs1, ys2 - ys1, zs2 - zs1]
    vca = [xs3 - xs1, ys3 - ys1, zs3 - zs1]
    ev31 = vba[1] * vca[2] - vba[2] * vca[1]
    ev32 = vba[2] * vca[0] - vba[0] * vca[2]
    ev33 = vba[0] * vca[1] - vba[1] * vca[0]
    rr = np.sqrt(ev31 * ev31 + ev32 * ev32 + ev33 * ev33)
    ev31, ev32, ev33 = ev31 / rr, ev32 / rr, ev33 / rr
    vert = np.abs(ev33) < 1.0
    ev11 = np.where(vert, -ev32, 1.0)
    ev12 = np.where(vert, ev31, 0.0)
    ev13 = np.zeros_like(ev31)
    rr = np.sqrt(ev11 * ev11 + ev12 * ev12)
    ev11 = np.where(vert, ev11 / rr, 1.0)
    ev12 = np.where(vert, ev12 / rr, 0.0)
    ev21 = ev32 * ev13 - ev33 * ev12
    ev22 = ev33 * ev11 - ev31 * ev13
    ev23 = ev31 * ev12 - ev32 * ev11
    t1 = vba[0] * vba[0] + vba[1] * vba[1] + vba[2] * vba[2]
    t2 = vca[0] * vca[0] + vca[1] * vca[1] + vca[2] * vca[2]
    t3 = vba[0] * vca[0] + vba[1] * vca[1] + vba[2] * vca[2]
    ds = 0.5 * np.sqrt(t1 * t2 - t3 * t3)
    return ev11, ev12, ev13, ev21, ev22, ev23, ev31, ev32, ev33, ds


def write_stl(path, tri):
    """tri: (n, 3, 3) vertices.  7 lines per facet, as the reference counts them."""
    with open(path, "w") as f:
        f.write("solid fault\n")
        for t in tri:
            f.write("facet normal 0 0 0\n outer loop\n")
            for v in t:
                f.write(f"  vertex {v[0]:.17g} {v[1]:.17g} {v[2]:.17g}\n")
            f.write(" endloop\nendfacet\n")
        f.write("endsolid fault\n")


def read_stl(path):
    """The reference's .stl reader: facet count = lines/7, vertices in order."""
    with open(path) as f:
        lines = f.read().splitlines()
    n = len(lines) // 7
    start = next(i for i, l in enumerate(lines) if l.split() and l.split()[0] == "facet")
    xs = np.zeros((3, n)); ys = np.zeros((3, n)); zs = np.zeros((3, n))
    p = start + 1
    for k in range(n):
        p += 1  # outer loop
        for v in range(3):
            w = lines[p].split()
            xs[v, k], ys[v, k], zs[v, k] = float(w[1]), float(w[2]), float(w[3])
            p += 1
        p += 3  # endloop, endfacet, facet
    return xs, ys, zs


def rough_fault(nx, nz, length, width, hurst=0.8, amp_ratio=1e-3, seed=0):
    """Seeded self-affine rough vertical strike-slip surface, 2*nx*nz triangles.

    Fault plane x in [0, length] along strike, z in [-width, 0]; the
    out-of-plane offset y(x,z) is a random field with power spectrum
    ~ k^-(2H+2) scaled so that the RMS amplitude over wavelength `length` is
    amp_ratio.  Returns tri (n,3,3).
    """
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx + 1, d=length / nx)
    kz = np.fft.fftfreq(nz + 1, d=width / nz)
    K = np.sqrt(kx[:, None] ** 2 + kz[None, :] ** 2)
    K[0, 0] = np.inf
    spec = K ** (-(hurst + 1.0)) * np.exp(2j * np.pi * rng.random(K.shape))
    field = np.real(np.fft.ifft2(spec))
    field -= field.mean()
    field *= amp_ratio * length / max(field.std(), 1e-300)
    x = np.linspace(0.0, length, nx + 1)
    z = np.linspace(0.0, -width, nz + 1)
    tri = np.zeros((2 * nx * nz, 3, 3))
    t = 0
    for i in range(nx):
        for j in range(nz):
            p00 = (x[i], field[i, j], z[j])
            p10 = (x[i + 1], field[i + 1, j], z[j])
            p01 = (x[i], field[i, j + 1], z[j + 1])
            p11 = (x[i + 1], field[i + 1, j + 1], z[j + 1])
            tri[t] = (p00, p01, p10); t += 1
            tri[t] = (p10, p01, p11); t += 1
    return tri


def tri_geometry(tri):
    """Vertex arrays, collocation points and ev frames of a triangle list."""
    xs = tri[:, :, 0].T.copy(); ys = tri[:, :, 1].T.copy(); zs = tri[:, :, 2].T.copy()
    xcol = (xs[0] + xs[1] + xs[2]) / 3
    ycol = (ys[0] + ys[1] + ys[2]) / 3
    zcol = (zs[0] + zs[1] + zs[2]) / 3
    ev = evcalc(xs[0], xs[1], xs[2], ys[0], ys[1], ys[2], zs[0], zs[1], zs[2])
    g = dict(xcol=xcol, ycol=ycol, zcol=zcol, xs1=xs[0], xs2=xs[1], xs3=xs[2], ys1=ys[0], ys2=ys[1], ys3=ys[2],
             zs1=zs[0], zs2=zs[1], zs3=zs[2])
    for name, a in zip(("ev11", "ev12", "ev13", "ev21", "ev22", "ev23", "ev31", "ev32", "ev33"), ev[:9]):
        g[name] = a
    return g, ev[9]
