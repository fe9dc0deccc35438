"""Model fields built on the device from cell-centred order parameters (ae_op_set_model_mixture,
ae_op_set_model_degraded) against the oracle's restatements, through the operator they feed:
Fapply with the device-built stiffness must match the oracle's Fapply with the oracle-built one
to 1e-12 of the field's max-norm, and the mixed eigenstrain the oracle's to 1e-13."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300._lib import AeError
from anisotropicfracture_gb300.elastic import Elastic, Field, level_desc
from helpers import bc_random, normwise_err
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("memory", ["host", "device"])
def test_mixture_matches_oracle(memory):
    """Three cubic phases with eigenstrains (PhaseFieldMicrostructure's Affine::Cubic mixture)."""
    n = 12
    rng = np.random.default_rng(401)
    L = po.level(n)
    eta_lo = (-1, -1, 0)
    eta = 0.05 + rng.random((3, n + 1, n + 2, n + 2))
    table = models.cubic(1.68, 1.21, 0.75, models.random_rotations(3, rng))
    F0table = 0.01 * rng.standard_normal((3, 9))
    C_ref, F0_ref = po.model_mixture((0, 0, 0), (n, n, n), eta, eta_lo, table, F0table)

    op = Elastic([level_desc(n)], models.MAJORMINOR)
    if memory == "host":
        F0 = np.zeros((9,) + L.shape)
        op.SetModelMixture(0, Field(eta, eta_lo), table, F0table, Field(F0))
    else:
        F0d = torch.zeros((9,) + L.shape, dtype=torch.float64, device="cuda")
        op.SetModelMixture(0, Field(dev(eta), eta_lo), table, F0table, Field(F0d))
        F0 = host(F0d)
    assert normwise_err(F0, F0_ref) <= 1e-13
    bc = bc_random(rng)
    op.SetBC(bc)
    op.SetUniform(False)
    op.prepareForSolve()
    u = rng.standard_normal((3,) + L.shape)
    f = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(u)))
    assert normwise_err(host(f), po.fapply(L, models.MAJORMINOR, C_ref, bc.type, u)) <= TOL64


def test_degraded_two_levels_matches_oracle():
    """PolymerDegradation's isotropic degradation on a coarse level and a refined patch: the
    patch's two ghost layers keep the undamaged stiffness, which Fapply reads at the patch edge."""
    rng = np.random.default_rng(402)
    Ls = po.amr_levels(8, 2)
    lam0, mu0 = 2.0, 1.0
    op = Elastic([level_desc(tuple(L.dom_hi), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx)) for L in Ls],
                 models.ISOTROPIC)
    Cs = []
    for a, L in enumerate(Ls):
        slo = tuple(L.lo[d] - L.ng for d in range(3))
        shi = tuple(L.hi[d] + L.ng for d in range(3))
        eta_lo = tuple(L.lo[d] - 1 for d in range(3))
        eta = 0.9 * rng.random((2,) + tuple(L.hi[d] - L.lo[d] + 2 for d in (2, 1, 0)))
        Cs.append(po.model_degraded(slo, shi, tuple(L.lo), tuple(L.hi), eta, eta_lo, lam0, mu0))
        op.SetModelDegraded(a, Field(eta, eta_lo), lam0, mu0)
    bc = bc_random(rng)
    op.SetBC(bc)
    op.SetUniform(False)
    op.prepareForSolve()
    for a, L in enumerate(Ls):
        lo = tuple(L.lo[d] - L.ng for d in range(3))
        u = rng.standard_normal((3,) + L.shape)
        f = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
        op.Fapply(a, 0, Field(f, lo), Field(dev(u), lo))
        ref = po.fapply(L, models.ISOTROPIC, Cs[a], bc.type, u)
        g = L.ng
        v = (slice(None),) + ((slice(g, -g),) * 3 if g else (slice(None),) * 3)
        assert normwise_err(host(f)[v], ref[v]) <= TOL64, "amrlev %d" % a


def test_builders_report_bad_order_parameters():
    n = 6
    op = Elastic([level_desc(n)], models.ISOTROPIC)
    with pytest.raises(AeError):  # the phases sum to zero: the reference divides by zero
        op.SetModelMixture(0, Field(np.zeros((2, n + 1, n + 2, n + 2)), (-1, -1, 0)), np.ones((2, 2)))
    with pytest.raises(AeError):  # a cell mean above 1: the reference aborts
        op.SetModelDegraded(0, Field(np.full((1, n + 2, n + 2, n + 2), 1.5), (-1, -1, -1)), 1.0, 1.0)
    with pytest.raises(AeError):  # eta does not cover the cells the nodes read
        op.SetModelDegraded(0, Field(np.full((1, n, n, n), 0.5), (0, 0, 0)), 1.0, 1.0)
    mm = Elastic([level_desc(n)], models.MAJORMINOR)
    with pytest.raises(AeError):  # degradation is defined for the isotropic model only
        mm.SetModelDegraded(0, None, 1.0, 1.0)
    # a valid call afterwards replaces the stiffness
    op.SetModelDegraded(0, Field(np.full((1, n + 2, n + 2, n + 2), 0.5), (-1, -1, -1)), 4.0, 2.0)
    op.prepareForSolve()
