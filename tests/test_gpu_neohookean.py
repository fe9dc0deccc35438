"""Newton<NeoHookean> on the GPU (finite kinematics, the 45-slot Sym::Major tangent):
ae_newton_neohookean's right-hand side and tangent stiffness, ae_neohookean_dw's DW and W, and
whole Newton solves, against the oracle (oracle/pyoracle.py: neohookean_newton_residual,
neohookean_newton, the ORC_MAJOR operator; the oracle's NeoHookean and its Sym::Major operator are
pinned to the reference's own code in tests/test_golden_ref.py).

Tolerances (FP64): the right-hand side, DW, W and the tangent operator's Fapply within 1e-12 of
the field's max-norm; per node within 1e-11 of max(|ref_node|, 1e-3 max|ref|) (the GPU takes
det F and F^-T from cofactors, the oracle from numpy's LU: the tangent's slots differ in their
last bits before any stencil sums them).  Newton solves end at the converged discrete solution;
GPU and oracle, each solving every correction to 1e-12, agree to 1e-9 of max|u|."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300.elastic import FACES, BCElastic, Elastic, Field, Newton, level_desc
from helpers import bc_random, normwise_err, pernode_err
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MU, KAPPA = 1.3, 2.7
NEO = models.NeoHookean(MU, KAPPA)
TOL = 1e-12
TOL_NODE = 1e-11


def _desc(L):
    return level_desc(tuple(L.dom_hi[d] for d in range(3)), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx))


def _lo(L):
    return tuple(L.lo[d] - L.ng for d in range(3))


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _close(got, ref, what):
    assert normwise_err(got, ref) < TOL, what
    assert pernode_err(got, ref) < TOL_NODE, what


def _small_field(rng, L, amp):
    """A displacement whose gradient stays well inside J > 0."""
    return amp * rng.standard_normal((3,) + L.shape)


@pytest.mark.parametrize("fine", [False, True])
def test_rhs_and_tangent_match_oracle(fine):
    rng = np.random.default_rng(21 + fine)
    Ls = po.amr_levels(8, 2) if fine else [po.level((9, 8, 7), dx=(0.11, 0.125, 0.14))]
    a = len(Ls) - 1
    L = Ls[a]
    bc = bc_random(rng)
    u = _small_field(rng, L, 0.01)
    b = rng.standard_normal((3,) + L.shape)
    rhs_ref, ddw = po.neohookean_newton_residual(L, MU, KAPPA, bc.type, u, b)
    C45 = po.major45(ddw)
    op = Elastic([_desc(Lk) for Lk in Ls], models.MAJOR)
    if fine:  # the coarse level needs a stiffness too: the small-strain tangent everywhere
        c0 = po.major45(po.neohookean_ddw(np.eye(3), MU, KAPPA))[:, None, None, None]
        op.SetModel(0, Field(np.ascontiguousarray(np.broadcast_to(c0, (45,) + Ls[0].shape))))
    op.SetBC(bc)
    rd = _dev(b.copy())
    op.NewtonNeoHookean(a, Field(rd, _lo(L)), Field(_dev(u), _lo(L)), Field(_dev(b), _lo(L)), NEO)
    _close(_host(rd), rhs_ref, "Newton right-hand side")
    # host fabs take the staged path and give the same values
    rh = b.copy()
    op.NewtonNeoHookean(a, Field(rh, _lo(L)), Field(u, _lo(L)), Field(b, _lo(L)), NEO)
    assert np.array_equal(rh, _host(rd))
    # the level's stiffness is now DDW(I + grad u): its operator is the oracle's Sym::Major one
    op.SetUniform(False)
    op.prepareForSolve()
    v = rng.standard_normal((3,) + L.shape)
    f = torch.zeros_like(_dev(v))
    op.Fapply(a, 0, Field(f, _lo(L)), Field(_dev(v), _lo(L)))
    _close(_host(f), po.fapply(L, po.ORC_MAJOR, C45, bc.type, v), "tangent Fapply")
    dg = torch.zeros_like(f)
    op.Diagonal(a, 0, Field(dg, _lo(L)))
    _close(_host(dg), po.diagonal(L, po.ORC_MAJOR, C45, bc.type), "tangent Diagonal")
    op.close()


def test_dw_and_w_match_oracle():
    rng = np.random.default_rng(5)
    L = po.level((7, 6, 8))
    u = _small_field(rng, L, 0.03)
    # grad u with Newton::DW's domain stencils: DW of a Diagonal model of ones is grad u itself
    g, _ = po.newton_dw(L, po.ORC_DIAGONAL, np.ones((9,) + L.shape), u)
    F = np.moveaxis(g, 0, -1).reshape(L.shape + (3, 3)) + np.eye(3)
    dw_ref = np.moveaxis(po.neohookean_dw(F, MU, KAPPA).reshape(L.shape + (9,)), -1, 0)
    w_ref = po.neohookean_w(F, MU, KAPPA)
    op = Elastic([_desc(L)], models.MAJOR)
    dw = torch.zeros((9,) + L.shape, dtype=torch.float64, device="cuda")
    w = torch.zeros((1,) + L.shape, dtype=torch.float64, device="cuda")
    op.NeoHookeanDW(0, Field(_dev(u)), NEO, dw=Field(dw), w=Field(w))
    _close(_host(dw), dw_ref, "DW")
    assert normwise_err(_host(w)[0], w_ref) < TOL
    # the Newton mirror's DW / W with the model give the same fields
    dw2, w2 = torch.zeros_like(dw), torch.zeros_like(w)
    s = Newton(op)
    s.DW([Field(dw2)], [Field(_dev(u))], model=NEO)
    s.W([Field(w2)], [Field(_dev(u))], model=NEO)
    assert torch.equal(dw2, dw) and torch.equal(w2, w)
    op.close()


def _uniaxial(L, d):
    """Symmetry rollers on the low faces, x = 1 pulled to 1 + d, the rest traction-free."""
    bc = BCElastic()
    for f, name in enumerate(FACES):
        for p, ax in enumerate("XYZ"):
            bc.type[f, p] = BCElastic.Traction
            if ax + "LO" in name:
                bc.type[f, p] = BCElastic.Displacement
            elif ax == "X" and "XHI" in name:
                bc.type[f, p], bc.val[f, p] = BCElastic.Displacement, d
    return bc


def _newton(Ls, bc, b, nriters, precision="fp64", u0=None):
    op = Elastic([_desc(L) for L in Ls], models.MAJOR)
    op.SetBC(bc)
    op.SetUniform(False)
    s = Newton(op)
    s.setNRIters(nriters)
    s.setPrecision(precision)
    s.setPreSmooth(2)
    s.setPostSmooth(2)
    us = [np.zeros_like(bk) if u0 is None else u0[k].copy() for k, bk in enumerate(b)]
    s.solve([Field(x, _lo(L)) for x, L in zip(us, Ls)], [Field(bk, _lo(L)) for bk, L in zip(b, Ls)],
            model=NEO, tol_rel=1e-12, tol_abs=0.0)
    op.close()
    return us


def test_uniaxial_stretch_known_answer():
    """The exact solution is homogeneous, F = diag(s, t, t) with P_yy(F) = 0, and the nodal
    operator reproduces affine fields exactly, so Newton must land on it."""
    from scipy.optimize import brentq
    d = 0.1
    s = 1.0 + d
    t = brentq(lambda t: po.neohookean_dw(np.diag([s, t, t]), MU, KAPPA)[1, 1], 0.5, 1.5)
    L = po.level(4)
    bc = _uniaxial(L, d)
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    u = _newton([L], bc, [b], 7)[0]
    X, Y, Z = po.node_coords(L)
    exact = np.stack([(s - 1) * X, (t - 1) * Y, (t - 1) * Z])
    assert np.abs(u - exact).max() < 1e-9


@pytest.fixture(scope="module")
def random_load():
    """A random nodal load and a pulled face on a 12 x 10 x 8-cell block, and three oracle Newton
    iterations from zero.  The tangent operator (C : grad grad u + grad C : grad u) is not the
    exact derivative of the discrete residual (central differences of DW), so away from affine
    fields the iteration converges linearly, in the reference as here."""
    rng = np.random.default_rng(8)
    L = po.level((12, 10, 8), dx=(1.0 / 12, 1.0 / 10, 1.0 / 8))
    bc = _uniaxial(L, 0.05)
    b = po.bc_init(L, bc.type, bc.val, 0.2 * rng.standard_normal((3,) + L.shape))
    ref, hist = po.neohookean_newton(L, MU, KAPPA, bc.type, np.zeros_like(b), b, nriters=3, tol_rel=1e-12,
                                     max_fmg_iter=100000000, bottom=1, nu1=2, nu2=2)
    assert hist[-1] < 0.1 * hist[0]
    return L, bc, b, ref


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_matches_oracle_on_a_random_load(random_load, precision):
    """Three Newton iterations on the GPU and in the oracle from the same start."""
    L, bc, b, ref = random_load
    got = _newton([L], bc, [b], 3, precision)[0]
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_two_level_uniaxial_stretch():
    """Newton<NeoHookean> on an AMR hierarchy (a refined patch inside the domain), the tangent
    set on every level each iteration: the homogeneous uniaxial solution on both levels."""
    from scipy.optimize import brentq
    d = 0.05
    s = 1.0 + d
    t = brentq(lambda t: po.neohookean_dw(np.diag([s, t, t]), MU, KAPPA)[1, 1], 0.5, 1.5)
    Ls = po.amr_levels(8, 2)
    bc = _uniaxial(Ls[0], d)
    bs = [po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape)) for L in Ls]
    us = _newton(Ls, bc, bs, 6)
    for L, u in zip(Ls, us):
        X, Y, Z = po.node_coords(L)
        exact = np.stack([(s - 1) * X, (t - 1) * Y, (t - 1) * Z])
        v = tuple(slice(L.ng, L.ng + L.hi[d] - L.lo[d] + 1) for d in (2, 1, 0))
        assert np.abs(u[(slice(None),) + v] - exact[(slice(None),) + v]).max() < 1e-9


def test_major_kind_rejects_linear_model_calls():
    from anisotropicfracture_gb300._lib import AeError
    L = po.level(4)
    op = Elastic([_desc(L)], models.MAJOR)
    u = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    sig = torch.zeros((9,) + L.shape, dtype=torch.float64, device="cuda")
    with pytest.raises(AeError):
        op.Stress(0, Field(sig), Field(u))
    with pytest.raises(AeError):
        op.SetModelGrains(0, Field(np.zeros((1,) + L.shape, np.int32)), np.ones((1, 45)))
    op.close()
    op2 = Elastic([_desc(L)], models.ISOTROPIC)
    op2.SetBC(BCElastic())
    with pytest.raises(AeError):
        op2.NewtonNeoHookean(0, Field(u.clone()), Field(u), Field(u.clone()), NEO)
    op2.close()
