"""The small single-level workload at full size on the GPU, against the oracle's full solve.

64^3 cells (65^3 nodes), unit cube, isotropic sphere inclusion (centre 0.5, radius 0.25, E 10 /
nu 0.3 inside, E 1 / nu 0.3 outside; the 2-cell diffuse interface of IC::Ellipse, because a sharp
10:1 jump makes the reference's damped-Jacobi smoother diverge), u = 0 on z = 0, u = (0, 0, 0.01)
on z = 1, traction-free lateral faces; V-cycle with one pre and one post smoother call of two
damped-Jacobi sweeps (Operator.cpp:109), CG bottom solve, 1e-8 relative residual.

Checks, through the C ABI:
- the FP64 GPU solve takes the oracle's iteration count (+-1) and lands within 1e-8 (normwise)
  of the oracle's solution;
- the mixed-precision solve lands within 1e-7 of the oracle's solution taken to 1e-10;
- the oracle recomputes b - A x for every GPU solution: its max-norm meets the solve's target;
- Fapply / Fsmooth / residual at this size match the oracle to 1e-12 per node (floor 1e-3 of the
  field's max-norm, helpers.pernode_err) and 1e-12 normwise.
"""
import numpy as np
import pytest

from anisotropicfracture_gb300 import microstructure, models
from anisotropicfracture_gb300.elastic import Elastic, Field, Linear, level_desc
from helpers import bc_pull_z, normwise_err, pernode_err, pernode_report
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = 64
TOL64 = 1e-12


@pytest.fixture(scope="module")
def problem():
    L = po.level(N)
    Cf = microstructure.sphere_inclusion_iso((0, 0, 0), (N, N, N), (1.0 / N,) * 3)
    bc = bc_pull_z()
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    ref, st, rc = po.solve(L, po.ORC_ISOTROPIC, Cf, bc.type, np.zeros_like(b), b, 1e-8, 0.0,
                           max_fmg_iter=0, bottom=0, nu1=1, nu2=1)
    assert rc == 0 and st.converged
    tight, st_t, rc_t = po.solve(L, po.ORC_ISOTROPIC, Cf, bc.type, ref, b, 1e-10, 0.0,
                                 max_fmg_iter=0, bottom=0, nu1=1, nu2=1)
    assert rc_t == 0
    return dict(L=L, Cf=Cf, bc=bc, b=b, ref=ref, st=st, tight=tight)


def gpu_solve(p, precision, inner=1):
    op = Elastic([level_desc(N)], models.ISOTROPIC)
    op.SetModel(0, Field(p["Cf"]))
    op.SetBC(p["bc"])
    op.SetUniform(False)
    s = Linear(op)
    s.setMaxFmgIter(0)
    s.setBottomSolver("cg")
    s.setPreSmooth(1)
    s.setPostSmooth(1)
    s.setPrecision(precision)
    s.opts.inner_cycles = inner
    x = np.zeros_like(p["b"])
    s.solve(Field(x), Field(p["b"]), 1e-8, 0.0)
    return x, s.stats, op


def oracle_residual(p, x):
    _, rn = po.residual(p["L"], po.ORC_ISOTROPIC, p["Cf"], p["bc"].type, x, p["b"])
    return rn


def test_config0_fp64_matches_oracle(problem):
    x, st, op = gpu_solve(problem, "fp64")
    assert st.converged
    assert abs(st.iters - problem["st"].iters) <= 1, (st.iters, problem["st"].iters)
    assert normwise_err(x, problem["ref"]) <= 1e-8
    assert normwise_err(x, problem["tight"]) <= 1e-7
    rn = oracle_residual(problem, x)
    assert rn <= st.target * (1 + 1e-6), (rn, st.target)
    print("config0 fp64: iters %d (oracle %d), err vs oracle %.2e, vs tight %.2e, oracle residual %.3e / target %.3e"
          % (st.iters, problem["st"].iters, normwise_err(x, problem["ref"]), normwise_err(x, problem["tight"]),
             rn, st.target))


@pytest.mark.parametrize("inner", [1, 12])
def test_config0_mixed_matches_oracle(problem, inner):
    """inner = FP32 V-cycles per FP64 residual (the benchmark runs 12)."""
    x, st, op = gpu_solve(problem, "mixed", inner)
    assert st.converged
    err = normwise_err(x, problem["tight"])
    assert err <= 1e-7, err
    rn = oracle_residual(problem, x)
    assert rn <= st.target * (1 + 1e-6), (rn, st.target)
    print("config0 mixed (%d inner): iters %d, cycles %d, err vs tight oracle %.2e, oracle residual %.3e / target %.3e"
          % (inner, st.iters, st.cycles, err, rn, st.target))


def test_config0_operators_per_node(problem):
    L, Cf, bc = problem["L"], problem["Cf"], problem["bc"]
    op = Elastic([level_desc(N)], models.ISOTROPIC)
    op.SetModel(0, Field(Cf))
    op.SetBC(bc)
    op.SetUniform(False)
    op.prepareForSolve()
    rng = np.random.default_rng(64)
    u = rng.standard_normal((3,) + L.shape)
    b = rng.standard_normal((3,) + L.shape)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    f = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(u)))
    torch.cuda.synchronize()
    ref_f = po.fapply(L, po.ORC_ISOTROPIC, Cf, bc.type, u)
    xd = dev(u)
    op.Fsmooth(0, 0, Field(xd), Field(dev(b)), 2, 2.0 / 3.0)
    torch.cuda.synchronize()
    D = po.diagonal(L, po.ORC_ISOTROPIC, Cf, bc.type)
    ref_s = po.fsmooth(L, po.ORC_ISOTROPIC, Cf, bc.type, D, u, b, 2, 2.0 / 3.0)
    r = torch.zeros_like(f)
    op.Residual(0, 0, Field(r), Field(dev(u)), Field(dev(b)))
    torch.cuda.synchronize()
    ref_r, _ = po.residual(L, po.ORC_ISOTROPIC, Cf, bc.type, u, b)
    for name, got, ref in (("fapply", f, ref_f), ("fsmooth", xd, ref_s), ("residual", r, ref_r)):
        g = got.cpu().numpy()
        print("config0 %s per-node relative error by floor: %s" % (name, pernode_report(g, ref)))
        assert normwise_err(g, ref) <= TOL64, name
        assert pernode_err(g, ref) <= TOL64, name
