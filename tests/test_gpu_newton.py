"""Newton<T> on the GPU: the Newton right-hand side, DW and W against the oracle (FP64, 1e-12 of
the field's max-norm), host and device fabs, and an eigenstrain (Affine model) Newton solve."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300.elastic import Elastic, Field, Newton, level_desc
from helpers import bc_pull_z, bc_random, normwise_err, random_coeffs
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


def _desc(L):
    return level_desc(tuple(L.dom_hi[d] for d in range(3)), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx))


def _lo(L):
    return tuple(L.lo[d] - L.ng for d in range(3))


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("model", [models.ISOTROPIC, models.MAJORMINOR])
@pytest.mark.parametrize("fine", [False, True])
@pytest.mark.parametrize("affine", [False, True])
def test_newton_residual_matches_oracle(model, fine, affine):
    rng = np.random.default_rng(10 + model + 2 * fine + 4 * affine)
    # a refined patch with ghost nodes (AMR level 1 of a two-level operator), or a single level
    Ls = po.amr_levels(8, 2) if fine else [po.level((9, 8, 7))]
    a = len(Ls) - 1
    L = Ls[a]
    Cs = [random_coeffs(model, Lk.shape, rng) for Lk in Ls]
    Cf = Cs[a]
    bc = bc_random(rng)
    u = rng.standard_normal((3,) + L.shape)
    b = rng.standard_normal((3,) + L.shape)
    F0 = 0.1 * rng.standard_normal((9,) + L.shape) if affine else None
    ref = po.newton_residual(L, model, Cf, bc.type, u, b, F0=F0)
    op = Elastic([_desc(Lk) for Lk in Ls], model)
    for k, Lk in enumerate(Ls):
        op.SetModel(k, Field(Cs[k], _lo(Lk)))
    op.SetBC(bc)
    rd = _dev(b.copy())
    op.NewtonResidual(a, Field(rd, _lo(L)), Field(_dev(u), _lo(L)), Field(_dev(b), _lo(L)),
                      Field(_dev(F0), _lo(L)) if affine else None)
    torch.cuda.synchronize()
    assert normwise_err(rd.cpu().numpy(), ref) < TOL
    # host fabs take the staged path and give the same values
    rh = b.copy()
    op.NewtonResidual(a, Field(rh, _lo(L)), Field(u, _lo(L)), Field(b, _lo(L)),
                      Field(np.ascontiguousarray(F0), _lo(L)) if affine else None)
    assert np.array_equal(rh, rd.cpu().numpy())
    op.close()


@pytest.mark.parametrize("model", [models.ISOTROPIC, models.MAJORMINOR])
def test_newton_dw_and_w_match_oracle(model):
    rng = np.random.default_rng(3)
    L = po.level((7, 6, 8))
    Cf = random_coeffs(model, L.shape, rng)
    u = rng.standard_normal((3,) + L.shape)
    op = Elastic([_desc(L)], model)
    op.SetModel(0, Field(Cf))
    for F0 in (None, 0.05 * rng.standard_normal((9,) + L.shape)):
        dw_ref, w_ref = po.newton_dw(L, model, Cf, u, F0=F0)
        dw, w = torch.zeros((9,) + L.shape, dtype=torch.float64, device="cuda"), torch.zeros(
            (1,) + L.shape, dtype=torch.float64, device="cuda")
        op.NewtonDW(0, Field(_dev(u)), Field(dw), Field(w), Field(_dev(F0)) if F0 is not None else None)
        torch.cuda.synchronize()
        assert normwise_err(dw.cpu().numpy(), dw_ref) < TOL
        assert normwise_err(w.cpu().numpy()[0], w_ref) < TOL
    op.close()


def test_eigenstrain_newton_solve_matches_oracle():
    """An isotropic cube with a spherical eigenstrain inclusion (Affine::Isotropic, the Eshelby
    set-up): one Newton iteration from u = 0, GPU against the oracle's N(u) + Linear solve."""
    n = 16
    L = po.level(n)
    lam, mu = models.lame_from_E_nu(1.0, 0.3)
    Cf = np.ascontiguousarray(np.stack([np.full(L.shape, lam), np.full(L.shape, mu)]))
    X, Y, Z = po.node_coords(L)
    inside = ((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2) < 0.2 ** 2
    F0 = np.zeros((9,) + L.shape)
    for q in (0, 4, 8):
        F0[q] = 0.01 * inside
    bc = bc_pull_z()
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    rhs = po.newton_residual(L, po.ORC_ISOTROPIC, Cf, bc.type, np.zeros_like(b), b, F0=F0)
    ref, st, rc = po.solve(L, po.ORC_ISOTROPIC, Cf, bc.type, np.zeros_like(b), rhs, 1e-10, 0.0, bottom=0, nu1=2,
                           nu2=2)
    assert rc == 0
    op = Elastic([_desc(L)], models.ISOTROPIC)
    op.SetModel(0, Field(Cf))
    op.SetBC(bc)
    op.SetUniform(False)
    s = Newton(op)
    s.setMaxFmgIter(0)
    s.opts.bottom, s.opts.nu1, s.opts.nu2 = 0, 2, 2
    u = np.zeros_like(b)
    s.solve([Field(u)], [Field(b)], tol_rel=1e-10, tol_abs=0.0, F0=[Field(np.ascontiguousarray(F0))])
    assert s.stats.converged
    assert np.abs(u - ref).max() / np.abs(ref).max() < 1e-8
    op.close()
