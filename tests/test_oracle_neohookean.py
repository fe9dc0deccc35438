"""The oracle's restatement of Model::Solid::Elastic::NeoHookean (W, DW, DDW;
src/Model/Solid/Elastic/NeoHookean.H:19-66), the finite-kinematics model of the Newton path:
DW is the derivative of W and DDW the derivative of DW (central differences), DDW has major
symmetry, and at F = I the tangent is the isotropic tensor with bulk modulus kappa and shear
modulus mu."""
import numpy as np

from oracle import pyoracle as po

MU, KAPPA = 1.3, 2.7


def random_F(rng, n):
    return np.eye(3) + 0.2 * rng.standard_normal((n, 3, 3))


def test_dw_is_the_derivative_of_w():
    rng = np.random.default_rng(1)
    F = random_F(rng, 8)
    dw = po.neohookean_dw(F, MU, KAPPA)
    h = 1e-6
    for k in range(3):
        for l in range(3):
            E = np.zeros((3, 3))
            E[k, l] = h
            fd = (po.neohookean_w(F + E, MU, KAPPA) - po.neohookean_w(F - E, MU, KAPPA)) / (2 * h)
            assert np.allclose(dw[:, k, l], fd, rtol=1e-6, atol=1e-8)


def test_ddw_is_the_derivative_of_dw_and_major_symmetric():
    rng = np.random.default_rng(2)
    F = random_F(rng, 8)
    ddw = po.neohookean_ddw(F, MU, KAPPA)
    h = 1e-6
    for k in range(3):
        for l in range(3):
            E = np.zeros((3, 3))
            E[k, l] = h
            fd = (po.neohookean_dw(F + E, MU, KAPPA) - po.neohookean_dw(F - E, MU, KAPPA)) / (2 * h)
            assert np.allclose(ddw[:, :, :, k, l], fd, rtol=1e-6, atol=1e-8)
    assert np.allclose(ddw, np.einsum("nijkl->nklij", ddw), rtol=1e-13, atol=1e-13)


def test_small_strain_limit_is_isotropic():
    I = np.eye(3)
    assert abs(po.neohookean_w(I, MU, KAPPA)) < 1e-15
    assert np.abs(po.neohookean_dw(I, MU, KAPPA)).max() < 1e-15
    lam = KAPPA - 2.0 * MU / 3.0
    iso = (lam * np.einsum("ij,kl->ijkl", I, I)
           + MU * (np.einsum("ik,jl->ijkl", I, I) + np.einsum("il,jk->ijkl", I, I)))
    assert np.allclose(po.neohookean_ddw(I, MU, KAPPA), iso, rtol=1e-14, atol=1e-14)


def test_residual_from_dw_reproduces_the_linear_newton_residual():
    """For Linear::Isotropic the residual from a DW field evaluated outside the oracle
    (sigma = lambda tr(grad u) I + mu (grad u + grad u^T)) equals the oracle's own."""
    from helpers import bc_random
    rng = np.random.default_rng(3)
    L = po.level((8, 6, 10))
    lam, mu = 1.7, 0.9
    C = np.stack([np.full(L.shape, lam), np.full(L.shape, mu)])
    bc = bc_random(rng)
    u = rng.standard_normal((3,) + L.shape)
    b = rng.standard_normal((3,) + L.shape)
    g = np.moveaxis(po.newton_grad(L, u), 0, -1).reshape(L.shape + (3, 3))
    sig = lam * np.trace(g, axis1=-2, axis2=-1)[..., None, None] * np.eye(3) + mu * (g + np.swapaxes(g, -1, -2))
    dw = np.ascontiguousarray(np.moveaxis(sig.reshape(L.shape + (9,)), -1, 0))
    ref = po.newton_residual(L, po.ORC_ISOTROPIC, C, bc.type, u, b)
    got = po.newton_residual_dw(L, bc.type, u, b, dw)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_neohookean_residual_small_displacement_limit():
    """For displacements of size s the NeoHookean residual's operator part N(u) equals the
    linear isotropic one (lambda = kappa - 2 mu / 3) up to O(s^2)."""
    from helpers import bc_random
    rng = np.random.default_rng(4)
    L = po.level(8)
    bc = bc_random(rng)
    bc.type[:] = np.where(bc.type == 0, 1, bc.type)  # traction / Neumann rows: N(u) involves DW
    s = 1e-6
    u = s * rng.standard_normal((3,) + L.shape)
    zero = np.zeros((3,) + L.shape)
    neo, ddw = po.neohookean_newton_residual(L, MU, KAPPA, bc.type, u, zero)
    C = np.stack([np.full(L.shape, KAPPA - 2 * MU / 3), np.full(L.shape, MU)])
    lin = po.newton_residual(L, po.ORC_ISOTROPIC, C, bc.type, u, zero)
    assert np.abs(neo - lin).max() <= 1e-4 * np.abs(lin).max()
    assert ddw.shape == L.shape + (3, 3, 3, 3)


def test_neohookean_homogeneous_deformation_is_in_equilibrium_inside():
    """u = A x gives a uniform F and DW: div DW = 0 at every interior node."""
    L = po.level(6)
    A = np.array([[0.05, 0.01, -0.02], [0.0, -0.03, 0.01], [0.02, 0.0, 0.04]])
    X, Y, Z = po.node_coords(L)
    x = np.stack([X, Y, Z])
    u = np.einsum("pd,d...->p...", A, x)
    b = np.zeros_like(u)
    rhs, _ = po.neohookean_newton_residual(L, MU, KAPPA, np.zeros((26, 3), np.int32), u, b)
    assert np.abs(rhs[:, 1:-1, 1:-1, 1:-1]).max() < 1e-12


def iso_tensor(lam, mu):
    I = np.eye(3)
    return (lam[..., None, None, None, None] * np.einsum("ij,kl->ijkl", I, I)
            + mu[..., None, None, None, None] * (np.einsum("ik,jl->ijkl", I, I) + np.einsum("il,jk->ijkl", I, I)))


def test_major_kind_reproduces_the_isotropic_operator():
    """The 45-slot Sym::Major kind, filled with the isotropic tensor node by node, gives the
    isotropic operator's Fapply and Diagonal (∇C term and BC rows included)."""
    from helpers import bc_random
    rng = np.random.default_rng(5)
    L = po.level((8, 6, 10))
    lam = 1.0 + rng.random(L.shape)
    mu = 0.5 + rng.random(L.shape)
    Ciso = np.ascontiguousarray(np.stack([lam, mu]))
    C45 = po.major45(iso_tensor(lam, mu))
    assert C45.shape == (45,) + L.shape
    bc = bc_random(rng)
    u = rng.standard_normal((3,) + L.shape)
    ref = po.fapply(L, po.ORC_ISOTROPIC, Ciso, bc.type, u)
    got = po.fapply(L, po.ORC_MAJOR, C45, bc.type, u)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    dref = po.diagonal(L, po.ORC_ISOTROPIC, Ciso, bc.type)
    dgot = po.diagonal(L, po.ORC_MAJOR, C45, bc.type)
    assert np.abs(dgot - dref).max() <= 1e-13 * np.abs(dref).max()


def test_major45_layout_is_the_reference_table():
    """Spot checks of the slot table of Matrix4<3, Sym::Major>::operator() (Matrix4_Major.H:203-258):
    slot 1 holds C_0001 = C_0100, slot 11 C_0110 = C_1001, slot 24 C_1010, slot 44 C_2222."""
    T = np.zeros((3, 3, 3, 3))
    for idx, v in [((0, 0, 0, 1), 1.0), ((0, 1, 1, 0), 2.0), ((1, 0, 1, 0), 3.0), ((2, 2, 2, 2), 4.0)]:
        T[idx] = v
        T[idx[2], idx[3], idx[0], idx[1]] = v
    c = po.major45(T)
    assert (c[1], c[11], c[24], c[44]) == (1.0, 2.0, 3.0, 4.0)
    assert np.count_nonzero(c) == 4


def test_neohookean_newton_uniaxial_known_answer():
    """Uniaxial stretch of a NeoHookean block with symmetry rollers on the low faces, x = 1 pulled
    to 1 + d and the rest traction-free: the exact solution is homogeneous, F = diag(s, t, t) with
    P_yy(F) = 0, and the nodal operator reproduces affine fields exactly, so Newton must land on
    it, with the corrections falling quadratically."""
    from scipy.optimize import brentq
    from anisotropicfracture_gb300.elastic import FACES
    D_, T_ = 0, 1
    d = 0.1
    s = 1.0 + d
    t = brentq(lambda t: po.neohookean_dw(np.diag([s, t, t]), MU, KAPPA)[1, 1], 0.5, 1.5)
    L = po.level(4)
    bt = np.full((26, 3), T_, np.int32)
    bv = np.zeros((26, 3))
    for f, name in enumerate(FACES):
        for p, ax in enumerate("XYZ"):
            if ax + "LO" in name:
                bt[f, p] = D_
            elif ax == "X" and "XHI" in name:
                bt[f, p], bv[f, p] = D_, d
    b = po.bc_init(L, bt, bv, np.zeros((3,) + L.shape))
    u, hist = po.neohookean_newton(L, MU, KAPPA, bt, np.zeros_like(b), b, nriters=7, tol_rel=1e-12,
                                   max_fmg_iter=100000000, bottom=1, nu1=2, nu2=2)
    X, Y, Z = po.node_coords(L)
    exact = np.stack([(s - 1) * X, (t - 1) * Y, (t - 1) * Z])
    assert np.abs(u - exact).max() < 1e-9
    assert hist[3] < 1e-6 and hist[-1] < 1e-10
    assert hist[2] < hist[1] ** 1.5 * 10  # quadratic convergence, loosely
