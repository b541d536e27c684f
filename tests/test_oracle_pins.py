"""Pins of the CPU oracle against known answers that do not depend on it.

The reference cannot be compiled here (Fortran + MPI, no compiler), so these
are the oracle's anchors: two independent published formulations must agree
(Okada's rectangle vs two Nikkhoo-Walter triangles; Okada's long vertical
strike-slip fault vs the 2D antiplane closed form), plus algorithmic identities
of ACA+ and of the matvec.
"""
import math

import numpy as np
import pytest

MU = LAM = 32.04
ALPHA = 2.0 / 3.0  # (lambda+mu)/(lambda+2mu) for nu = 0.25


def okada_stress(O, x, y, z, d1, d2, dip=90.0, depth=5.0, al=(-1, 1), aw=(-0.5, 0.5), full=True):
    u = O.okada(ALPHA, x, y, z, depth, dip, al[0], al[1], aw[0], aw[1], d1, d2, 0.0, fullspace=full)
    uxx, uyx, uzx, uxy, uyy, uzy, uxz, uyz, uzz = u[3:]
    exx, eyy, ezz = uxx, uyy, uzz
    exy, eyz, ezx = .5 * (uxy + uyx), .5 * (uyz + uzy), .5 * (uzx + uxz)
    tr = exx + eyy + ezz
    return np.array([LAM * tr + 2 * MU * exx, LAM * tr + 2 * MU * eyy, LAM * tr + 2 * MU * ezz,
                     2 * MU * exy, 2 * MU * ezx, 2 * MU * eyz])


@pytest.mark.parametrize("pt", [(0.3, 0.7, -5.2), (2.5, -1.0, -3.0), (-0.4, 0.05, -4.9), (0.0, 3.0, -8.0)])
@pytest.mark.parametrize("slip", [(1, 0), (0, 1)])
def test_okada_equals_two_triangles(oracle, pt, slip):
    """A uniform-slip rectangle equals the two triangles that tile it."""
    A, B, C, D = (-1, 0, -5.5), (1, 0, -5.5), (1, 0, -4.5), (-1, 0, -4.5)
    so = okada_stress(oracle, *pt, *slip)
    st = (oracle.tdstressfs(*pt, A, B, C, slip[0], slip[1], 0, MU, LAM)
          + oracle.tdstressfs(*pt, A, C, D, slip[0], slip[1], 0, MU, LAM))
    assert np.max(np.abs(so - st)) <= 1e-12 * np.max(np.abs(so))


@pytest.mark.parametrize("dip", [30.0, 60.0, 90.0, 120.0])
@pytest.mark.parametrize("pt", [(0.3, 0.7, -3.2), (2.5, -1.0, -2.0), (0.0, 1.0, -0.3), (1.5, -0.5, -6.0)])
@pytest.mark.parametrize("slip", [(1, 0), (0, 1)])
def test_okada_half_space_equals_two_half_space_triangles(oracle, dip, pt, slip):
    """'3dht': Nikkhoo-Walter triangles in a half space (main + image
    dislocation + the free-surface correction of AngDisStrainFSC) tile Okada's
    half-space rectangle, close to the surface too (z = -0.3 km, where the
    full-space answer is off by order one)."""
    d, dep = math.radians(dip), 3.0
    cw = lambda e: (e * math.cos(d), -dep + e * math.sin(d))
    A, B, C, D = (-1, *cw(-0.5)), (1, *cw(-0.5)), (1, *cw(0.5)), (-1, *cw(0.5))
    so = okada_stress(oracle, *pt, *slip, dip=dip, depth=dep, full=False)
    st = (oracle.tdstresshs(*pt, A, B, C, slip[0], slip[1], 0, MU, LAM)
          + oracle.tdstresshs(*pt, A, C, D, slip[0], slip[1], 0, MU, LAM))
    assert np.max(np.abs(so - st)) <= 1e-12 * np.max(np.abs(so))


def test_half_space_triangle_leaves_the_surface_traction_free(oracle):
    """sigma_xz, sigma_yz, sigma_zz of '3dht' vanish on z = 0 for a buried
    triangle with mixed strike, dip and tensile slip."""
    P1, P2, P3 = (0, 0, -2), (2, 1, -3), (1, 2, -1.5)
    for pt in [(0.5, 0.5, 0.0), (3, -2, 0.0), (-1, 4, 0.0), (8, 3, 0.0)]:
        s = oracle.tdstresshs(*pt, P1, P2, P3, 1, 0.5, 0.2, MU, LAM)
        deep = oracle.tdstresshs(pt[0], pt[1], -1.0, P1, P2, P3, 1, 0.5, 0.2, MU, LAM)
        assert max(abs(s[2]), abs(s[4]), abs(s[5])) <= 1e-13 * np.max(np.abs(deep)), pt


def test_okada_long_fault_is_2d_antiplane(oracle):
    """A very long vertical strike-slip rectangle in a half space reproduces the
    2D antiplane half-space kernel of '2dvs' (matels2dpa_ij minus its image)."""
    n, ds0 = 64, 0.5
    xel, xer, xcol, _ = oracle.mesh_2dp(n, ds0)
    g = oracle.Geometry(oracle.ORC_2DVS, n, "s", xcol=xcol, xel=xel, xer=xer)
    L = 3.0e4  # long enough that the finite-length error (~L^-2) is below 1e-6, short enough for FP64
    for (i, j) in [(10, 10), (10, 11), (3, 40), (50, 7), (1, 64)]:
        e2d = oracle.entry(g, i, j)
        # source: depth interval [xel_j, xer_j] on the plane y=0; receiver at depth xcol_i
        w = xer[j - 1] - xel[j - 1]
        u = oracle.okada(ALPHA, 0.0, 0.0, -xcol[i - 1], xer[j - 1], 90.0, -L, L, 0.0, w, 1.0, 0.0, 0.0,
                         fullspace=False)
        sxy = MU * (u[6] + u[4])  # 2 mu e_xy
        # same magnitude; the 2D kernel's sign convention is opposite to Okada's disl1
        assert abs(sxy / e2d + 1.0) <= 2e-6, (i, j, sxy, e2d)


def _geometry_2d(oracle, problem, v, xel, xer, yel, yer):
    from hbi_gb300 import mesh
    xel, xer, yel, yer, xcol, ycol, ang, _ = mesh.mesh_2dn(xel, xer, yel, yer)
    n = len(xel)
    return oracle.Geometry(problem, n, v, xcol=xcol, ycol=ycol, zcol=np.zeros(n), xel=xel, xer=xer, yel=yel,
                           yer=yer, ang=ang)


def test_2dph_free_surface_is_traction_free(oracle):
    """Edge dislocations of '2dph' (D2dip2) leave the free surface y = 0
    traction free: receivers on y = 0 with horizontal planes (ang = 0) feel
    neither shear nor normal traction, whatever the source."""
    from hbi_gb300 import mesh
    src = mesh.bent_fault_2d(8, 4.0, 1.5, 40.0, seed=1)
    m = 7
    xs = np.linspace(-4, 8, m)
    xel = np.concatenate([xs - 0.05, src[0]]); xer = np.concatenate([xs + 0.05, src[1]])
    yel = np.concatenate([np.zeros(m), src[2]]); yer = np.concatenate([np.zeros(m), src[3]])
    for v in "sn":
        g = _geometry_2d(oracle, oracle.ORC_2DPH, v, xel, xer, yel, yer)
        at_depth = max(abs(oracle.entry(g, m + k, m + k)) for k in range(1, 9))
        for i in range(1, m + 1):
            for j in range(m + 1, m + 9):
                assert abs(oracle.entry(g, i, j)) <= 1e-13 * at_depth, (v, i, j)


def test_2dph_deep_is_2dn_full_space(oracle):
    """Far below the free surface the half-space edge dislocations of '2dph'
    (D2dip2) reduce to the full-space plane-strain kernel of '2dn'
    (tensor2d_ij, written with vs / vp instead of nu): the two formulations
    agree for shear and normal traction on a bent fault 2000 km deep (the
    image's share is ~(L / 4000 km)^2 = 1e-6).  The two prefactors differ by
    the rounding of the constants: mu/(2 pi (1-nu)) with nu = 0.25 against
    mu (1 - vs^2/vp^2)/pi with vs = 3.464 (not sqrt(12)) and vp = 6."""
    from hbi_gb300 import mesh
    ends = mesh.bent_fault_2d(40, 4.0, 2000.0, 35.0, seed=2, rough=0.3)
    prefactor_ratio = (1 - (3.464 / 6.0) ** 2) * 2 * (1 - 0.25)
    for v in "sn":
        gh = _geometry_2d(oracle, oracle.ORC_2DPH, v, *ends)
        gf = _geometry_2d(oracle, oracle.ORC_2DN, v, *ends)
        A = np.array([[oracle.entry(gh, i, j) for j in range(1, 41)] for i in range(1, 41)])
        B = np.array([[oracle.entry(gf, i, j) for j in range(1, 41)] for i in range(1, 41)]) / prefactor_ratio
        assert np.max(np.abs(A - B)) <= 5e-6 * np.max(np.abs(B)), v


def test_tdstress_symmetry_and_decay(oracle):
    """Stress from a triangle is symmetric under reflecting the receiver
    through the triangle plane (normal-parallel shear flips) and decays as r^-3."""
    P1, P2, P3 = (0, 0, -1), (1, 0, -1), (0, 0, 0)
    far1 = oracle.tdstressfs(30, 20, -10, P1, P2, P3, 1, 0, 0, MU, LAM)
    far2 = oracle.tdstressfs(60, 40, -20, P1, P2, P3, 1, 0, 0, MU, LAM)
    ratio = np.max(np.abs(far1)) / np.max(np.abs(far2))
    assert 7.5 < ratio < 8.5


def test_aca_recovers_block_and_matvec(oracle):
    """ACA+ with eps=1e-6 reproduces the dense 2dvs operator; H*1 matches A*1."""
    n, ds0 = 512, 40.0 / 512
    xel, xer, xcol, _ = oracle.mesh_2dp(n, ds0)
    g = oracle.Geometry(oracle.ORC_2DVS, n, "s", xcol=xcol, xel=xel, xer=xer)
    coord = np.stack([xcol, np.zeros(n), np.zeros(n)], 1)
    lod, leaves, cnt = oracle.build_structure(coord)
    assert cnt == len(leaves)
    p = oracle.default_params()
    p[70] = 1e-6
    H = oracle.HMatrix(g, lod, leaves, p)
    A = oracle.dense_matrix(g, lod)
    assert np.linalg.norm(H.to_dense() - A) <= 1e-9 * np.linalg.norm(A)
    u = np.ones(n)
    assert np.linalg.norm(H.matvec(u) - A @ u) <= 1e-7 * np.linalg.norm(A @ u)
    # the OpenMP matvec (reference thread ranges, atomic accumulation) agrees
    assert np.allclose(H.matvec(u, nthreads=4), H.matvec(u), rtol=1e-13, atol=1e-13 * np.abs(H.matvec(u)).max())


def test_single_precision_literals(oracle):
    """Cash-Karp and rkqs constants carry the reference's default-real values."""
    a, b, c, dc = oracle.cashkarp()
    assert b[1] == float(np.float32(3.0) / np.float32(40.0))
    assert c[0] == float(np.float32(37.0) / np.float32(378.0))
    assert dc[5] == float(np.float32(512.0) / np.float32(1771.0)) - 0.25
    k = oracle.rkqs_consts()
    assert k[0] == float(np.float32(0.9)) and k[3] == float(np.float32(1e-20))
    assert abs(sum(c) - 1.0) < 1e-7  # the fifth-order weights sum to one (to single precision)


def test_rkqs_relaxes_to_steady_sliding(oracle):
    """A velocity-strengthening fault loaded at the plate rate stays at V = vpl."""
    n = 128
    ds0 = 40.0 / n
    xel, xer, xcol, _ = oracle.mesh_2dp(n, ds0)
    g = oracle.Geometry(oracle.ORC_2DVS, n, "s", xcol=xcol, xel=xel, xer=xer)
    coord = np.stack([xcol, np.zeros(n), np.zeros(n)], 1)
    lod, leaves, _ = oracle.build_structure(coord)
    p = oracle.default_params(); p[70] = 1e-6
    H = oracle.HMatrix(g, lod, leaves, p)
    a, b, f0, sig, v0 = 0.015, 0.010, 0.6, 50.0, 1e-9
    vref = float(np.float32(1e-6))
    psi = f0 - b * math.log(v0 / vref)
    tau = a * sig * math.asinh(v0 / (2 * vref) * math.exp(psi / a))
    y = np.tile([a * math.log(2 * vref / v0 * math.sinh(tau / sig / a)), tau, sig], n)
    # perturb the state: an exactly steady state has errmax = 0 <= tiny, which
    # the reference's controller rejects until the step underflows
    y[1::3] *= 1.0 + 1e-3 * np.sin(np.arange(n))
    R = oracle.RSF(n, H, a=np.full(n, a), b=np.full(n, b), dc=np.full(n, 0.01), f0=np.full(n, f0),
                   vplv=np.full(n, v0))
    x, h = 0.0, 1.0
    for _ in range(60):
        rc, y, x, hdid, h, em, nr = R.rkqs(y, x, h, 1e-6)
        assert rc == 0
    V = 2 * vref * np.exp(-y[0::3] / a) * np.sinh(y[1::3] / y[2::3] / a)
    assert np.allclose(V, v0, rtol=1e-3), (x, V.min(), V.max())


def test_mlp_oracle_gradient_matches_finite_differences(oracle):
    """The proposer's forward/backward restatement (the checker of the GPU
    training kernels) against central differences of its own loss."""
    nin, h, B = 3, 4, 16
    rng = np.random.default_rng(1)
    npar = h * nin + h + h * h + h + h + 1
    p = (0.5 * rng.standard_normal(npar)).astype(np.float32)
    x = rng.standard_normal((B, nin)).astype(np.float32)
    t = rng.standard_normal(B).astype(np.float32)
    loss, g, _ = oracle.mlp_loss_grad(nin, h, p, x, t)
    step = 1e-2
    fd = np.zeros(npar)
    for k in range(npar):
        pp, pm = p.copy(), p.copy()
        pp[k] += step
        pm[k] -= step
        fd[k] = (oracle.mlp_loss_grad(nin, h, pp, x, t)[0] - oracle.mlp_loss_grad(nin, h, pm, x, t)[0]) / (
            float(pp[k]) - float(pm[k]))
    assert np.allclose(g, fd, rtol=2e-2, atol=2e-4)


def test_mlp_oracle_pinball_gradient_matches_finite_differences(oracle):
    """The same for the pinball (quantile) loss: away from the kinks (no
    sample's residual within the finite-difference step of zero) its
    gradient is the central difference of the loss."""
    nin, h, B, tau = 3, 4, 16, 0.2
    rng = np.random.default_rng(4)
    npar = h * nin + h + h * h + h + h + 1
    p = (0.5 * rng.standard_normal(npar)).astype(np.float32)
    x = rng.standard_normal((B, nin)).astype(np.float32)
    t = rng.standard_normal(B).astype(np.float32) + 3.0
    loss, g, out = oracle.mlp_loss_grad(nin, h, p, x, t, tau)
    r = out - t
    assert np.all(np.abs(r) > 0.5)
    assert loss == pytest.approx(np.mean(np.where(r > 0, (1 - tau) * r, -tau * r)), rel=1e-6)
    step = 1e-2
    fd = np.zeros(npar)
    for k in range(npar):
        pp, pm = p.copy(), p.copy()
        pp[k] += step
        pm[k] -= step
        fd[k] = (oracle.mlp_loss_grad(nin, h, pp, x, t, tau)[0] - oracle.mlp_loss_grad(nin, h, pm, x, t, tau)[0]) / (
            float(pp[k]) - float(pm[k]))
    assert np.allclose(g, fd, rtol=2e-2, atol=2e-4)


def test_proposer_labels_recover_the_ideal_step():
    """training_set's label is the step that would have met the target error
    under Cash-Karp's h**5 error law."""
    from hbi_gb300 import proposer
    rng = np.random.default_rng(2)
    n = 50
    rows = []
    hstar = 10.0 ** rng.uniform(1, 3, n)
    hnext = hstar * 10.0 ** rng.uniform(-0.3, 0.3, n)
    # step k+1 is first tried at h1 = hnext[k] (the rkqs proposal of step k)
    # with error e1 = E_TARGET (h1/hstar)**5; a rejected first try is
    # followed by an accepted retry at hstar
    acc = [(hstar[0], proposer.E_TARGET)]
    for k in range(1, n):
        h1 = hnext[k - 1]
        e1 = proposer.E_TARGET * (h1 / hstar[k]) ** 5
        acc.append((h1, e1) if e1 < 1.0 else (hstar[k], proposer.E_TARGET))
    for k in range(n):
        if k > 0:
            h1 = hnext[k - 1]
            e1 = proposer.E_TARGET * (h1 / hstar[k]) ** 5
            if e1 >= 1.0:
                rows.append([k + 1, 0.0, h1, e1, 0, 1e-9, 0.0, 0])
        rows.append([k + 1, 0.0, acc[k][0], acc[k][1], 1, 1e-9, hnext[k], 0])
    X, T = proposer.training_set(np.array(rows))
    assert X.shape[1] == 7 and len(T) == n - 3
    assert np.allclose(T, np.log10(hstar[3:n] / hnext[2:n - 1]), atol=1e-5)
