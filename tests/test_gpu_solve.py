"""GPU multigrid solves through ae_solve vs the CPU oracle's MLMG restatement, the
reference's known-answer solves on the GPU, mixed precision, and error behaviour."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, microstructure, models
from anisotropicfracture_gb300._lib import AeError
from anisotropicfracture_gb300.elastic import BCElastic, Elastic, Field, Linear, level_desc
from helpers import bc_pull_z, bc_uniaxial_x, normwise_err, random_coeffs
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def sphere_inclusion_problem(n):
    """n^3 cells: isotropic sphere inclusion (E 10 / 1, nu 0.3), pulled along z."""
    L = po.level(n)
    Cf = microstructure.sphere_inclusion_iso((0, 0, 0), (n, n, n), (1.0 / n,) * 3)
    bc = bc_pull_z()
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    return L, Cf, bc, b


def gpu_solver(n, model, Cf, bc, fmg=0, bottom=0, nu=1, precision="fp64", **kw):
    op = Elastic([level_desc(n)], model)
    op.SetModel(0, Field(Cf))
    op.SetBC(bc)
    op.SetUniform(False)
    s = Linear(op)
    s.setMaxFmgIter(fmg)
    s.opts.bottom = bottom
    s.opts.nu1 = s.opts.nu2 = nu
    s.setPrecision(precision)
    for k, v in kw.items():
        setattr(s.opts, k, v)
    return op, s


@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("fmg,bottom,nu", [(0, 0, 1), (100000000, 1, 2)])
def test_sphere_inclusion_fp64_matches_oracle(n, fmg, bottom, nu):
    L, Cf, bc, b = sphere_inclusion_problem(n)
    ref, st, rc = po.solve(L, po.ORC_ISOTROPIC, Cf, bc.type, np.zeros_like(b), b, 1e-8, 0.0,
                           max_fmg_iter=fmg, bottom=bottom, nu1=nu, nu2=nu)
    assert rc == 0
    op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc, fmg, bottom, nu)
    x = np.zeros_like(b)
    s.solve(Field(x), Field(b), 1e-8, 0.0)
    assert s.stats.converged
    assert abs(s.stats.iters - st.iters) <= 1
    assert s.stats.resfinal <= s.stats.target
    assert normwise_err(x, ref) < 1e-8


def test_sphere_inclusion_mixed_precision_error():
    """FP32 cycle inside FP64 refinement: 1e-8 residual, displacement within 1e-7 of the FP64 oracle."""
    n = 32
    L, Cf, bc, b = sphere_inclusion_problem(n)
    ref, st, rc = po.solve(L, po.ORC_ISOTROPIC, Cf, bc.type, np.zeros_like(b), b, 1e-10, 0.0)
    op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc, precision="mixed")
    x = np.zeros_like(b)
    s.solve(Field(x), Field(b), 1e-8, 0.0)
    assert s.stats.converged and s.stats.resfinal <= s.stats.target
    assert normwise_err(x, ref) < 1e-7


def test_polycrystal_fp64_and_mixed():
    n = 16
    L = po.level(n)
    Cf, gid, tab = microstructure.cubic_polycrystal((0, 0, 0), (n, n, n), (1.0 / n,) * 3, nseeds=8)
    bc = bc_pull_z()
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    ref, st, rc = po.solve(L, po.ORC_MAJORMINOR, Cf, bc.type, np.zeros_like(b), b, 1e-8, 0.0)
    assert rc == 0
    for prec, tol in (("fp64", 1e-8), ("mixed", 1e-7)):
        op, s = gpu_solver(n, models.MAJORMINOR, Cf, bc, precision=prec)
        x = np.zeros_like(b)
        s.solve(Field(x), Field(b), 1e-8, 0.0)
        assert s.stats.converged
        assert normwise_err(x, ref) < tol, prec


def test_trig_known_answer_on_gpu():
    """src/Test/Operator/Elastic_TrigTest.cpp through the GPU solve (2 % vs the sine series)."""
    n = 32
    L = po.level(n)
    xs = np.sin(np.pi * np.arange(n + 1) / n)
    S3 = xs[None, None, :] * xs[None, :, None] * xs[:, None, None]
    b = np.zeros((3,) + L.shape)
    b[0] = S3
    op, s = gpu_solver(n, models.DIAGONAL, np.ones((9,) + L.shape), BCElastic(), fmg=100000000, bottom=1, nu=2)
    x = np.zeros_like(b)
    s.solve(Field(x), Field(b), 1e-8, 1e-8)
    exact = -S3 / (3 * np.pi ** 2)
    assert np.abs(x[0] - exact).max() / np.abs(exact).max() < 0.02


def test_uniaxial_known_answer_on_gpu():
    """src/Test/Operator/Elastic_UniaxialTest.cpp through the GPU solve (1 %)."""
    n = 32
    L = po.level(n)
    bc = bc_uniaxial_x()
    Cf = np.empty((2,) + L.shape)
    Cf[0], Cf[1] = 6.0, 2.6
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    for prec in ("fp64", "mixed"):
        op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc, precision=prec)
        x = np.zeros_like(b)
        s.solve(Field(x), Field(b), 1e-8, 1e-8)
        exact = np.zeros_like(b)
        exact[0] = 0.1 * (np.arange(n + 1) / n)[None, None, :]
        err = sum(np.abs(x[c] - exact[c]).max() for c in range(3)) / 0.1
        assert err < 0.01, prec


def test_host_and_device_buffers_agree():
    n = 16
    L, Cf, bc, b = sphere_inclusion_problem(n)
    op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc)
    xh = np.zeros_like(b)
    s.solve(Field(xh), Field(b), 1e-8, 0.0)
    xd = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    s.solve(Field(xd), Field(torch.from_numpy(b).cuda()), 1e-8, 0.0)
    torch.cuda.synchronize()
    assert np.array_equal(xd.cpu().numpy(), xh)


def test_graph_and_eager_agree():
    n = 16
    L, Cf, bc, b = sphere_inclusion_problem(n)
    op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc, use_graph=1)
    xg = np.zeros_like(b)
    s.solve(Field(xg), Field(b), 1e-8, 0.0)
    s.opts.use_graph = 0
    xe = np.zeros_like(b)
    s.solve(Field(xe), Field(b), 1e-8, 0.0)
    assert np.array_equal(xg, xe)


def test_error_behaviour():
    n = 8
    L, Cf, bc, b = sphere_inclusion_problem(n)
    op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc, max_iter=1)
    x = np.zeros_like(b)
    with pytest.raises(AeError) as e:
        s.solve(Field(x), Field(b), 1e-12, 0.0)
    assert e.value.code == _lib.AE_ERR_NOT_CONVERGED
    bn = b.copy()
    bn[0, 3, 3, 3] = np.nan
    s.opts.max_iter = 50
    with pytest.raises(AeError) as e:
        s.solve(Field(np.zeros_like(b)), Field(bn), 1e-8, 0.0)
    assert e.value.code == _lib.AE_ERR_NAN
    # Fsmooth before the diagonal exists (Operator.cpp:105)
    op2 = Elastic([level_desc(n)], models.ISOTROPIC)
    op2.SetModel(0, Field(Cf))
    xd = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    with pytest.raises(AeError) as e:
        op2.Fsmooth(0, 0, Field(xd), Field(xd))
    assert e.value.code == _lib.AE_ERR_STATE
    # a field too small for the level is an argument error
    small = torch.zeros((3, 4, 4, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(AeError) as e:
        op.Fapply(0, 0, Field(small), Field(small))
    assert e.value.code == _lib.AE_ERR_ARG
    # NaN stiffness is reported by the diagonal (Elastic.cpp:347)
    Cn = Cf.copy()
    Cn[1, 2, 2, 2] = np.nan
    op3 = Elastic([level_desc(n)], models.ISOTROPIC)
    op3.SetModel(0, Field(Cn))
    with pytest.raises(AeError) as e:
        op3.prepareForSolve()
    assert e.value.code == _lib.AE_ERR_NAN


def test_fixed_iter_runs_exactly_that_many_iterations():
    """MLMG fixed_iter (Solver::Nonlocal::Linear::Parse, Linear.H:132-133): the solve stops after
    exactly that many iterations and reports no convergence failure; the iterate equals the one an
    ordinary solve has after as many iterations."""
    n = 16
    L, Cf, bc, b = sphere_inclusion_problem(n)
    op, s = gpu_solver(n, models.ISOTROPIC, Cf, bc)
    s.setFixedIter(3)
    x = np.zeros_like(b)
    s.solve(Field(x), Field(b), 1e-14, 0.0)
    assert s.stats.iters == 3 and not s.stats.converged
    op2, s2 = gpu_solver(n, models.ISOTROPIC, Cf, bc, max_iter=3)
    x2 = np.zeros_like(b)
    with pytest.raises(AeError):
        s2.solve(Field(x2), Field(b), 1e-14, 0.0)
    assert np.array_equal(x, x2)


@pytest.mark.parametrize("nlev", [1, 2])
def test_solveaffine_equals_solve_for_linear_models(nlev):
    """Linear::solveaffine (Linear.H:41-100) adds the negated apply of zero by the inhomogeneous
    operator to rhs inside the domain.  For the linear stiffness kinds that apply is exactly zero:
    the solution equals Linear::solve's bit for bit, and copyrhs writes back rhs unchanged."""
    from helpers import polycrystal_amr
    Ls, Cs, bc, bs = polycrystal_amr(16, nlev)
    lo = [tuple(L.lo[d] - L.ng for d in range(3)) for L in Ls]
    descs = [level_desc(tuple(L.dom_hi[d] for d in range(3)), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx))
             for L in Ls]
    out = []
    for affine in (False, True):
        op = Elastic(descs, models.MAJORMINOR)
        for a in range(nlev):
            op.SetModel(a, Field(Cs[a], lo[a]))
        op.SetBC(bc)
        op.SetUniform(False)
        s = Linear(op)
        s.setMaxFmgIter(0)
        xs = [np.zeros_like(b) for b in bs]
        rs = [b.copy() for b in bs]
        fx = [Field(x, l) for x, l in zip(xs, lo)]
        fr = [Field(r, l) for r, l in zip(rs, lo)]
        if affine:
            s.solveaffine(fx, fr, 1e-8, 0.0, copyrhs=True)
            for r, b in zip(rs, bs):
                assert np.array_equal(r, b)
        else:
            s.solve(fx, fr, 1e-8, 0.0)
        out.append((s.stats.iters, xs))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)
