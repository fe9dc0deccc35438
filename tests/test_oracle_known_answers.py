"""Pins the CPU oracle to the reference's own known-answer tests (restated, not copied)
and to independent restatements of its tables.  CPU only."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300.elastic import FACES
from helpers import D, N, T, bc_uniaxial_x, normwise_err, random_coeffs
from oracle import pyoracle as po


def _cos3(n):
    # IC::Trig2 with n = 1 on a unit box: cos(pi x / L) (src/IC/Trig2.H:86-95; L = 1,
    # src/Test/Numeric/Stencil.H:131)
    L = po.level(n)
    x = np.arange(n + 1) / n
    cx, sx = np.cos(np.pi * x), np.sin(np.pi * x)
    return L, x, cx, sx


def _interior(a):
    return a[..., 1:-1, 1:-1, 1:-1]


# ---------------------------------------------------------------- src/Test/Numeric/Stencil.H:58-106
@pytest.mark.parametrize("which", ["xx", "yy", "zz", "xy", "xz", "yz", "x", "y", "z"])
def test_stencil_derivatives_cos(which):
    """Stencil derivatives of cos(pi x) cos(pi y) cos(pi z) at 32^3 within 1 % (max-norm)."""
    n = 32
    L, x, cx, sx = _cos3(n)
    k = np.pi
    phi = cx[None, None, :] * cx[None, :, None] * cx[:, None, None]
    u = np.zeros((3,) + L.shape)
    u[0] = phi
    bct = np.zeros((26, 3), np.int32)
    if which in ("x", "y", "z"):
        eps = po.strain(L, u)  # eps_00 = d phi/dx, eps_01 = 0.5 d phi/dy, eps_02 = 0.5 d phi/dz
        comp = {"x": 0, "y": 1, "z": 2}[which]
        num = eps[comp] * (1.0 if comp == 0 else 2.0)
        ex = {"x": -k * sx[None, None, :] * cx[None, :, None] * cx[:, None, None],
              "y": -k * cx[None, None, :] * sx[None, :, None] * cx[:, None, None],
              "z": -k * cx[None, None, :] * cx[None, :, None] * sx[:, None, None]}[which]
        assert normwise_err(_interior(num[None])[0], _interior(ex[None])[0]) < 1e-2
        return
    if which in ("xx", "yy", "zz"):
        A = np.zeros(9)
        A[{"xx": 0, "yy": 1, "zz": 2}[which]] = 1.0  # f_0 = A_0j u_{0,jj}
        Cf = np.ascontiguousarray(np.broadcast_to(A[:, None, None, None], (9,) + L.shape))
        f = po.fapply(L, po.ORC_DIAGONAL, Cf, bct, u, uniform=True)[0]
        ex = -k * k * phi
    else:
        slot = {"xy": 1, "xz": 2, "yz": 7}[which]  # f_0 = 2 phi_{,ab} for a single nonzero slot
        a = np.zeros(21)
        a[slot] = 0.5
        Cf = np.ascontiguousarray(np.broadcast_to(a[:, None, None, None], (21,) + L.shape))
        f = po.fapply(L, po.ORC_MAJORMINOR, Cf, bct, u, uniform=True)[0]
        s = {"xy": (sx[None, None, :] * sx[None, :, None] * cx[:, None, None]),
             "xz": (sx[None, None, :] * cx[None, :, None] * sx[:, None, None]),
             "yz": (cx[None, None, :] * sx[None, :, None] * sx[:, None, None])}[which]
        ex = k * k * s
    assert normwise_err(_interior(f[None])[0], _interior(ex[None])[0]) < 1e-2


# ---------------------------------------------------------------- src/Test/Set/Matrix4.H:9-30
def test_majorminor_symmetry_and_slot_table():
    rng = np.random.default_rng(1)
    c21 = rng.random(21)
    C = models.full_from_slots(c21)
    assert np.array_equal(C, np.transpose(C, (2, 3, 0, 1)))  # major
    assert np.array_equal(C, np.transpose(C, (0, 1, 3, 2)))  # minor
    assert np.array_equal(C, np.transpose(C, (1, 0, 2, 3)))  # minor
    # two independent restatements of the uid -> slot map agree
    assert np.array_equal(po.mm_full(c21), C)
    # every slot is used, each by the expected number of index tuples (4 or 8 or 1/2)
    counts = np.bincount(models.SLOT.reshape(-1), minlength=21)
    assert counts.sum() == 81 and (counts > 0).all()


def test_majorminor_contractions_match_generic():
    """C:grad u and C:grad grad u of src/Set/Matrix4_MajorMinor.H:253-345 equal the
    generic 81-term contractions sigma_ij = C_ijkl g_kl and f_i = C_ijkl b_klj."""
    rng = np.random.default_rng(2)
    for _ in range(20):
        c21 = rng.standard_normal(21)
        C = models.full_from_slots(c21)
        g = rng.standard_normal((3, 3))
        b = rng.standard_normal((3, 3, 3))
        s = po.mm_stress(c21, g)
        assert np.allclose(s, np.einsum("ijkl,kl->ij", C, g), rtol=1e-13, atol=1e-13)
        f = po.mm_div(c21, b)
        assert np.allclose(f, np.einsum("ijkl,klj->i", C, b), rtol=1e-13, atol=1e-13)


def _cubic_define_loop(C11, C12, C44, R):
    """Literal restatement of src/Model/Solid/Linear/Cubic.H:37-58: Ctmp has C44 only where
    i == k and j == l, and each of the 21 slots keeps the value of the last (p,q,s,t)."""
    Ct = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    if i == j == k == l:
                        Ct[i, j, k, l] = C11
                    elif i == k and j == l:
                        Ct[i, j, k, l] = C44
                    elif i == j and k == l:
                        Ct[i, j, k, l] = C12
    out = np.zeros(21)
    for p in range(3):
        for q in range(3):
            for s in range(3):
                for t in range(3):
                    acc = 0.0
                    for i in range(3):
                        for j in range(3):
                            for k in range(3):
                                for l in range(3):
                                    acc += R[p, i] * R[s, k] * Ct[i, j, k, l] * R[q, j] * R[t, l]
                    out[models.SLOT[p, q, s, t]] = acc
    return out


def test_cubic_define_matches_reference_loop():
    """Linear::Cubic::Define: identity rotation puts C11/C12/C44 in the right slots; rotated
    tensors equal the reference's own assignment loop (including its slot-overwrite order)."""
    c = models.cubic(1.68, 1.21, 0.75, np.eye(3))
    Cf = models.full_from_slots(c)
    assert Cf[0, 0, 0, 0] == 1.68 and Cf[0, 0, 1, 1] == 1.21 and Cf[0, 1, 0, 1] == 0.75
    assert Cf[0, 0, 0, 1] == 0.0
    rng = np.random.default_rng(3)
    R = models.random_rotations(3, rng)
    assert np.allclose(np.einsum("gij,gkj->gik", R, R), np.eye(3)[None], atol=1e-14)
    assert np.allclose(np.linalg.det(R), 1.0)
    for g in range(3):
        assert np.allclose(models.cubic(1.68, 1.21, 0.75, R[g]), _cubic_define_loop(1.68, 1.21, 0.75, R[g]),
                           rtol=0, atol=1e-14)
    # a cubic symmetry operation (90 degrees about z) maps the tensor onto itself
    Rz = models.euler_rotation(0.0, np.pi / 2, 0.0)
    assert np.allclose(models.cubic(1.68, 1.21, 0.75, Rz), c, atol=1e-14)
    R1 = models.euler_rotation(0.3, 0.2, 0.1)
    assert np.allclose(R1 @ R1.T, np.eye(3))


# ---------------------------------------------------------------- src/Test/Operator/Elastic_TrigTest.cpp
@pytest.mark.parametrize("fmg,bottom", [(0, 0), (100000000, 1)])
def test_trig_solve(fmg, bottom):
    """Laplacian model, rhs sin(pi x) sin(pi y) sin(pi z) on component 0, displacement BCs:
    the solve matches -rhs / (3 pi^2) within 2 %."""
    n = 32
    L = po.level(n)
    x = np.arange(n + 1) / n
    s = np.sin(np.pi * x)
    S3 = s[None, None, :] * s[None, :, None] * s[:, None, None]
    b = np.zeros((3,) + L.shape)
    b[0] = S3
    bct, bcv = np.zeros((26, 3), np.int32), np.zeros((26, 3))
    b = po.bc_init(L, bct, bcv, b)
    Cf = np.ones((9,) + L.shape)
    nu = 2 if fmg else 1
    u, st, rc = po.solve(L, po.ORC_DIAGONAL, Cf, bct, np.zeros_like(b), b, 1e-8, 1e-8,
                         max_fmg_iter=fmg, bottom=bottom, nu1=nu, nu2=nu)
    assert rc == 0 and st.converged
    exact = -S3 / (3 * np.pi ** 2)
    assert np.abs(u[0] - exact).max() / np.abs(exact).max() < 0.02


# ---------------------------------------------------------------- src/Test/Operator/Elastic_UniaxialTest.cpp
@pytest.mark.parametrize("fmg,bottom", [(0, 0), (100000000, 1)])
def test_uniaxial_solve(fmg, bottom):
    """Isotropic mu = 2.6, lambda = 6.0, uniaxial displacement BCs: u_x = 0.1 x within 1 %."""
    n = 32
    L = po.level(n)
    bc = bc_uniaxial_x()
    Cf = np.empty((2,) + L.shape)
    Cf[0], Cf[1] = 6.0, 2.6
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    nu = 2 if fmg else 1
    u, st, rc = po.solve(L, po.ORC_ISOTROPIC, Cf, bc.type, np.zeros_like(b), b, 1e-8, 1e-8,
                         max_fmg_iter=fmg, bottom=bottom, nu1=nu, nu2=nu)
    assert rc == 0
    x = np.arange(n + 1) / n
    exact = np.zeros_like(b)
    exact[0] = 0.1 * x[None, None, :]
    err = sum(np.abs(u[c] - exact[c]).max() for c in range(3)) / sum(np.abs(exact[c]).max() for c in range(3))
    assert err < 0.01


# ---------------------------------------------------------------- src/Test/Operator/Elastic_RefluxTest.cpp
@pytest.mark.parametrize("m", [1.0, 2.0])
@pytest.mark.parametrize("nvec", [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (1, 1, 0)])
def test_fapply_affine_fields(m, nvec):
    """Fapply of the halfspace field alpha ((x - b).n)^m on component 1 (IC::Affine, b = (0, 0.25, 0))
    with uniform isotropic C (mu 2.6, lambda 6.0) equals the exact operator wherever the stencil
    does not straddle the kink: 0 for m = 1, 2 alpha [lambda n_1 n_i + mu (delta_i1 |n|^2 + n_i n_1)]
    for m = 2."""
    n = 32
    L = po.level(n)
    x, y, z = [np.arange(n + 1) / n] * 3
    X = np.meshgrid(z, y, x, indexing="ij")
    bvec = np.array([0.0, 0.25, 0.0])
    nv = np.array(nvec, dtype=float)
    val = (X[2] - bvec[0]) * nv[0] + (X[1] - bvec[1]) * nv[1] + (X[0] - bvec[2]) * nv[2]
    u = np.zeros((3,) + L.shape)
    u[1] = np.where(val >= 0, val ** m, 0.0)
    lam, mu = 6.0, 2.6
    Cf = np.empty((2,) + L.shape)
    Cf[0], Cf[1] = lam, mu
    f = po.fapply(L, po.ORC_ISOTROPIC, Cf, np.zeros((26, 3), np.int32), u)
    h = 1.0 / n
    safe = val > 2.5 * h * np.abs(nv).sum()
    safe[0, :, :] = safe[-1, :, :] = False
    safe[:, 0, :] = safe[:, -1, :] = False
    safe[:, :, 0] = safe[:, :, -1] = False
    if m == 1.0:
        exact = np.zeros(3)
    else:
        n2 = nv @ nv
        exact = 2 * (lam * nv[1] * nv + mu * (np.eye(3)[1] * n2 + nv * nv[1]))
    for i in range(3):
        assert np.allclose(f[i][safe], exact[i], rtol=1e-9, atol=1e-8)


# ---------------------------------------------------------------- BC classification and Init
def _classify_reference_chain(i, j, k, lo, hi):
    """Literal if-chain of src/BC/Operator/Elastic.H:140-167, face names as strings."""
    if i == lo and j == lo and k == lo: return "XLO_YLO_ZLO"
    if i == lo and j == lo and k == hi: return "XLO_YLO_ZHI"
    if i == lo and j == hi and k == lo: return "XLO_YHI_ZLO"
    if i == lo and j == hi and k == hi: return "XLO_YHI_ZHI"
    if i == hi and j == lo and k == lo: return "XHI_YLO_ZLO"
    if i == hi and j == lo and k == hi: return "XHI_YLO_ZHI"
    if i == hi and j == hi and k == lo: return "XHI_YHI_ZLO"
    if i == hi and j == hi and k == hi: return "XHI_YHI_ZHI"
    if j == lo and k == lo: return "YLO_ZLO"
    if j == lo and k == hi: return "YLO_ZHI"
    if j == hi and k == lo: return "YHI_ZLO"
    if j == hi and k == hi: return "YHI_ZHI"
    if k == lo and i == lo: return "ZLO_XLO"
    if k == lo and i == hi: return "ZLO_XHI"
    if k == hi and i == lo: return "ZHI_XLO"
    if k == hi and i == hi: return "ZHI_XHI"
    if i == lo and j == lo: return "XLO_YLO"
    if i == lo and j == hi: return "XLO_YHI"
    if i == hi and j == lo: return "XHI_YLO"
    if i == hi and j == hi: return "XHI_YHI"
    if i == lo: return "XLO"
    if i == hi: return "XHI"
    if j == lo: return "YLO"
    if j == hi: return "YHI"
    if k == lo: return "ZLO"
    if k == hi: return "ZHI"
    return None


@pytest.mark.parametrize("homogeneous", [False, True])
def test_bc_init_classification(homogeneous):
    n = 4
    L = po.level(n)
    rng = np.random.default_rng(5)
    bct = rng.choice([D, T, N], size=(26, 3)).astype(np.int32)
    bcv = rng.standard_normal((26, 3))
    rhs0 = rng.standard_normal((3,) + L.shape)
    rhs = po.bc_init(L, bct, bcv, rhs0, homogeneous)
    for k in range(n + 1):
        for j in range(n + 1):
            for i in range(n + 1):
                name = _classify_reference_chain(i, j, k, 0, n)
                if name is None:
                    assert np.array_equal(rhs[:, k, j, i], rhs0[:, k, j, i])
                    continue
                f = FACES.index(name)
                for d in range(3):
                    want = 0.0 if (homogeneous and bct[f, d] == D) else bcv[f, d]
                    assert rhs[d, k, j, i] == want


# ---------------------------------------------------------------- diagonal = probed diagonal
@pytest.mark.parametrize("model", [po.ORC_ISOTROPIC, po.ORC_MAJORMINOR, po.ORC_DIAGONAL])
def test_diagonal_matches_probe(model):
    """Elastic<T>::Diagonal (analytic) equals the self-coefficient probed with unit spikes,
    the generic Operator<Node>::Diagonal of src/Operator/Operator.cpp:33-88."""
    rng = np.random.default_rng(11)
    n = 6
    L = po.level(n)
    Cf = random_coeffs(model, L.shape, rng)
    bct = rng.choice([D, T, N], size=(26, 3)).astype(np.int32)
    Dg = po.diagonal(L, model, Cf, bct)
    nz, ny, nx = L.shape
    for (k, j, i) in [(0, 0, 0), (0, 3, 3), (3, 3, 3), (6, 6, 6), (2, 0, 6), (1, 2, 3), (6, 3, 0)]:
        for p in range(3):
            u = np.zeros((3,) + L.shape)
            u[p, k, j, i] = 1.0
            f = po.fapply(L, model, Cf, bct, u)
            assert np.isclose(f[p, k, j, i], Dg[p, k, j, i], rtol=1e-12, atol=1e-12)


def test_transfer_operators_exactness():
    """Full-weighting restriction keeps constants; trilinear interpolation reproduces
    trilinear fields exactly (src/Operator/Operator.cpp:454-624)."""
    n = 16
    Lf, Lc = po.level(n), po.coarsen(po.level(n))
    c = np.full((3,) + Lf.shape, 2.5)
    r = po.restrict(Lc, Lf, c)
    assert np.allclose(r, 2.5, rtol=0, atol=1e-14)
    xc = np.arange(n // 2 + 1) * (2.0 / n)
    Zc, Yc, Xc = np.meshgrid(xc, xc, xc, indexing="ij")
    lin = 1.0 + 2 * Xc - Yc + 0.5 * Zc + 0.25 * Xc * Yc * Zc
    crse = np.stack([lin, 2 * lin, -lin])
    fine = po.interp_add(Lf, Lc, np.zeros((3,) + Lf.shape), crse)
    xf = np.arange(n + 1) / n
    Zf, Yf, Xf = np.meshgrid(xf, xf, xf, indexing="ij")
    linf = 1.0 + 2 * Xf - Yf + 0.5 * Zf + 0.25 * Xf * Yf * Zf
    assert np.allclose(fine[0], linf, atol=1e-13) and np.allclose(fine[1], 2 * linf, atol=1e-13)


# ---------------------------------------------------------------- multi-level (src/test.cc:123-151)
def _amr_trig(nlev, n=32):
    Ls = po.amr_levels(n, nlev)
    bct, bcv = np.zeros((26, 3), np.int32), np.zeros((26, 3))
    bs, us, Cs, ex = [], [], [], []
    for L in Ls:
        X, Y, Z = po.node_coords(L)
        S3 = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
        b = np.zeros((3,) + L.shape)
        b[0] = S3
        bs.append(po.bc_init(L, bct, bcv, b))
        us.append(np.zeros_like(b))
        Cs.append(np.ones((9,) + L.shape))
        ex.append(-S3 / (3 * np.pi ** 2))
    return Ls, bct, bs, us, Cs, ex


def _valid(a, L):
    g = L.ng
    return a[(slice(None),) + (slice(g, a.shape[1] - g),) * 3] if g else a


@pytest.mark.parametrize("nlev", [2, 3])
def test_trig_solve_multilevel(nlev):
    """TrigTest on 2 and 3 AMR levels (each refining the central half): composite solve within 2 %."""
    Ls, bct, bs, us, Cs, ex = _amr_trig(nlev)
    u, st, rc = po.solve_amr(Ls, po.ORC_DIAGONAL, Cs, bct, us, bs, 1e-8, 1e-8, max_fmg_iter=0, bottom=0)
    assert rc == 0
    err = max(np.abs(_valid(u[a], L)[0] - _valid(ex[a][None], L)[0]).max() for a, L in enumerate(Ls))
    assert err / np.abs(ex[0]).max() < 0.02


@pytest.mark.parametrize("nlev", [2, 3])
def test_uniaxial_solve_multilevel(nlev):
    """UniaxialTest on 2 and 3 AMR levels within 1 %."""
    Ls = po.amr_levels(32, nlev)
    bc = bc_uniaxial_x()
    bs, us, Cs, ex = [], [], [], []
    for L in Ls:
        X, Y, Z = po.node_coords(L)
        c = np.empty((2,) + L.shape)
        c[0], c[1] = 6.0, 2.6
        bs.append(po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape)))
        us.append(np.zeros((3,) + L.shape))
        Cs.append(c)
        ex.append(0.1 * X)
    u, st, rc = po.solve_amr(Ls, po.ORC_ISOTROPIC, Cs, bc.type, us, bs, 1e-8, 1e-8)
    assert rc == 0
    err = max(np.abs(_valid(u[a], L)[0] - _valid(ex[a][None], L)[0]).max() for a, L in enumerate(Ls))
    assert err / 0.1 < 0.01
