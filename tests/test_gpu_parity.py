"""GPU operator kernels vs the CPU oracle on the same seeded inputs, through the C ABI.

Tolerance (FP64), both required:
- normwise: max|gpu - oracle| <= 1e-12 * max|oracle|;
- per node: |gpu - oracle| <= 1e-12 * max(|oracle_node|, 1e-3 * max|oracle|), i.e. relative to the
  node's own value wherever that is at least 1e-3 of the field's max-norm (helpers.pernode_err).
The kernels fuse multiply-adds that the oracle keeps separate, so nodes whose value comes from
cancelling much larger stencil terms differ in relative terms; the worst per-node error is printed
at the floors 0, 1e-9, 1e-6 and 1e-3.  FP32 kernels: 2e-5 of the max-norm."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300.elastic import BCElastic, Elastic, Field, level_desc
from helpers import bc_pull_z, bc_random, normwise_err, pernode_err, pernode_report, random_coeffs
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5
MODELS = [models.ISOTROPIC, models.MAJORMINOR, models.DIAGONAL]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def make_case(model, cells, bckind, uniform, seed, dx=None):
    rng = np.random.default_rng(seed)
    cells = (cells,) * 3 if np.isscalar(cells) else tuple(cells)
    L = po.level(cells, dx=dx)
    Cf = random_coeffs(model, L.shape, rng)
    bc = {"disp": BCElastic(), "pull_z": bc_pull_z(), "random": bc_random(rng)}[bckind]
    op = Elastic([level_desc(cells, dx=dx)], model)
    op.SetModel(0, Field(Cf))
    op.SetBC(bc)
    op.SetUniform(uniform)
    op.prepareForSolve()
    return rng, L, Cf, bc, op


CASES = [(m, n, bck, uni) for m in MODELS for (n, bck, uni) in
         [(8, "random", False), (9, "pull_z", False), (16, "random", True), ((8, 6, 10), "random", False)]]


@pytest.mark.parametrize("model,cells,bckind,uniform", CASES)
def test_fapply_matches_oracle(model, cells, bckind, uniform):
    dx = (0.1, 0.15, 0.08) if not np.isscalar(cells) else None
    rng, L, Cf, bc, op = make_case(model, cells, bckind, uniform, 100 + model, dx)
    u = rng.standard_normal((3,) + L.shape)
    f = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(u)))
    ref = po.fapply(L, model, Cf, bc.type, u, uniform)
    got = host(f)
    print("PERNODE fapply", model, cells, bckind, uniform, pernode_report(got, ref))
    assert normwise_err(got, ref) <= TOL64
    assert pernode_err(got, ref) <= TOL64


@pytest.mark.parametrize("model", MODELS)
def test_fapply_fp32_matches_oracle(model):
    rng, L, Cf, bc, op = make_case(model, 16, "random", False, 7)
    u = rng.standard_normal((3,) + L.shape)
    f = torch.zeros((3,) + L.shape, dtype=torch.float32, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(u.astype(np.float32))))
    ref = po.fapply(L, model, Cf, bc.type, u.astype(np.float32).astype(np.float64))
    assert normwise_err(host(f).astype(np.float64), ref) <= TOL32


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("bckind", ["random", "pull_z"])
def test_diagonal_all_levels(model, bckind):
    """Diagonal on every multigrid level; coarse stiffness from the oracle's restriction
    (averageDownCoeffsSameAmrLevel)."""
    rng, L, Cf, bc, op = make_case(model, 16, bckind, False, 21)
    Lm, Cm = L, Cf
    for m in range(op.NMGLevels(0)):
        if m > 0:
            Lc = po.coarsen(Lm)
            Cm = po.restrict(Lc, Lm, Cm)
            Lm = Lc
        Dg = torch.zeros((3,) + Lm.shape, dtype=torch.float64, device="cuda")
        op.Diagonal(0, m, Field(Dg))
        ref = po.diagonal(Lm, model, Cm, bc.type)
        got = host(Dg)
        print("PERNODE diagonal", model, bckind, m, pernode_report(got, ref))
        assert normwise_err(got, ref) <= TOL64, "mglev %d" % m
        assert pernode_err(got, ref) <= TOL64, "mglev %d" % m
        # coarse-level Fapply uses the restricted stiffness too
        u = rng.standard_normal((3,) + Lm.shape)
        f = torch.zeros_like(Dg)
        op.Fapply(0, m, Field(f), Field(dev(u)))
        assert normwise_err(host(f), po.fapply(Lm, model, Cm, bc.type, u)) <= TOL64


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("nsweeps", [1, 2])
def test_fsmooth_matches_oracle(model, nsweeps):
    rng, L, Cf, bc, op = make_case(model, 16, "pull_z", False, 31)
    x = rng.standard_normal((3,) + L.shape)
    b = rng.standard_normal((3,) + L.shape)
    xd = dev(x)
    op.Fsmooth(0, 0, Field(xd), Field(dev(b)), nsweeps, 2.0 / 3.0)
    Dg = po.diagonal(L, model, Cf, bc.type)
    ref = po.fsmooth(L, model, Cf, bc.type, Dg, x, b, nsweeps, 2.0 / 3.0)
    got = host(xd)
    print("PERNODE fsmooth", model, nsweeps, pernode_report(got, ref))
    assert normwise_err(got, ref) <= TOL64
    assert pernode_err(got, ref) <= TOL64


@pytest.mark.parametrize("model", MODELS)
def test_residual_and_norm(model):
    rng, L, Cf, bc, op = make_case(model, 12, "random", False, 41)
    x = rng.standard_normal((3,) + L.shape)
    b = rng.standard_normal((3,) + L.shape)
    r = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    nrm = op.Residual(0, 0, Field(r), Field(dev(x)), Field(dev(b)))
    ref, rn = po.residual(L, model, Cf, bc.type, x, b)
    got = host(r)
    print("PERNODE residual", model, pernode_report(got, ref))
    assert normwise_err(got, ref) <= TOL64
    assert pernode_err(got, ref) <= TOL64
    assert abs(nrm - rn) <= TOL64 * rn


def test_restriction_interpolation_bitwise():
    rng, L, Cf, bc, op = make_case(models.ISOTROPIC, 16, "disp", False, 51)
    Lc = po.coarsen(L)
    fine = rng.standard_normal((3,) + L.shape)
    crse = torch.zeros((3,) + Lc.shape, dtype=torch.float64, device="cuda")
    op.restriction(0, 1, Field(crse), Field(dev(fine)))
    assert normwise_err(host(crse), po.restrict(Lc, L, fine)) <= 1e-15
    c2 = rng.standard_normal((3,) + Lc.shape)
    f0 = rng.standard_normal((3,) + L.shape)
    fd = dev(f0)
    op.interpolation(0, 0, Field(fd), Field(dev(c2)))
    assert normwise_err(host(fd), po.interp_add(L, Lc, f0, c2)) <= 1e-15


@pytest.mark.parametrize("homogeneous", [False, True])
def test_bc_init(homogeneous):
    rng, L, Cf, bc, op = make_case(models.ISOTROPIC, 7, "random", False, 61)
    r0 = rng.standard_normal((3,) + L.shape)
    rd = dev(r0)
    op.BCInit(0, Field(rd), homogeneous)
    assert np.array_equal(host(rd), po.bc_init(L, bc.type, bc.val, r0, homogeneous))


@pytest.mark.parametrize("model", MODELS)
def test_strain_stress_energy(model):
    rng, L, Cf, bc, op = make_case(model, 10, "random", False, 71)
    u = rng.standard_normal((3,) + L.shape)
    ud = dev(u)
    for voigt in (False, True):
        e = torch.zeros((6 if voigt else 9,) + L.shape, dtype=torch.float64, device="cuda")
        op.Strain(0, Field(e), Field(ud), voigt)
        assert normwise_err(host(e), po.strain(L, u, voigt)) <= TOL64
        s = torch.zeros_like(e)
        op.Stress(0, Field(s), Field(ud), voigt)
        assert normwise_err(host(s), po.stress(L, model, Cf, u, voigt)) <= TOL64
    w = torch.zeros((1,) + L.shape, dtype=torch.float64, device="cuda")
    op.Energy(0, Field(w), Field(ud))
    assert normwise_err(host(w), po.energy(L, model, Cf, u)) <= TOL64


def test_fab_with_ghosts_and_offsets():
    """Fields may carry ghost nodes (AMReX fabs with nGrow = 2): the operator reads and
    writes through the fab's own box."""
    rng, L, Cf, bc, op = make_case(models.MAJORMINOR, 8, "pull_z", False, 81)
    u = rng.standard_normal((3,) + L.shape)
    ug = np.zeros((3, 13, 13, 13))
    ug[:, 2:-2, 2:-2, 2:-2] = u
    fg = torch.zeros((3, 13, 13, 13), dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(fg, lo=(-2, -2, -2)), Field(dev(ug), lo=(-2, -2, -2)))
    out = host(fg)
    ref = po.fapply(L, models.MAJORMINOR, Cf, bc.type, u)
    assert normwise_err(out[:, 2:-2, 2:-2, 2:-2], ref) <= TOL64
    assert np.all(out[:, :2] == 0) and np.all(out[:, -2:] == 0)


# ---------------------------------------------------------------- z-marching tiled kernels
@pytest.fixture
def tiled64(monkeypatch):
    """Operators created inside the test run their FP64 sweeps on the tiled kernels."""
    monkeypatch.setenv("AE_TILED64", "1")
    yield


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("cells,bckind,uniform", [(16, "random", False), (33, "pull_z", False),
                                                  ((40, 9, 20), "random", True)])
def test_tiled64_fapply_fsmooth(tiled64, model, cells, bckind, uniform):
    """The tiled kernel (FP64 instantiation) matches the oracle at 1e-12, including tile edges
    (domains that are not multiples of the tile) and the z-march boundaries."""
    rng, L, Cf, bc, op = make_case(model, cells, bckind, uniform, 300 + model)
    u = rng.standard_normal((3,) + L.shape)
    f = torch.zeros((3,) + L.shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(u)))
    assert normwise_err(host(f), po.fapply(L, model, Cf, bc.type, u, uniform)) <= TOL64
    b = rng.standard_normal((3,) + L.shape)
    xd = dev(u)
    op.Fsmooth(0, 0, Field(xd), Field(dev(b)), 2, 2.0 / 3.0)
    Dg = po.diagonal(L, model, Cf, bc.type)
    ref = po.fsmooth(L, model, Cf, bc.type, Dg, u, b, 2, 2.0 / 3.0, uniform)
    assert normwise_err(host(xd), ref) <= TOL64


@pytest.mark.parametrize("model", [models.ISOTROPIC, models.MAJORMINOR])
def test_tiled64_fine_patch_with_ghosts(tiled64, model):
    """Jacobi on an AMR patch with 2 ghost layers: ghost layer 1 updated, ring zeroed."""
    rng = np.random.default_rng(77)
    Ls = po.amr_levels(16, 2)
    Lf = Ls[1]
    Cs = [random_coeffs(model, L.shape, rng) for L in Ls]
    bc = bc_random(rng)
    descs = [level_desc(tuple(L.dom_hi), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx)) for L in Ls]
    op = Elastic(descs, model)
    for a, L in enumerate(Ls):
        op.SetModel(a, Field(Cs[a], tuple(L.lo[d] - L.ng for d in range(3))))
    op.SetBC(bc)
    op.SetUniform(False)
    op.prepareForSolve()
    lo = tuple(Lf.lo[d] - 2 for d in range(3))
    x = rng.standard_normal((3,) + Lf.shape)
    b = rng.standard_normal((3,) + Lf.shape)
    xd = dev(x)
    op.Fsmooth(1, 0, Field(xd, lo), Field(dev(b), lo), 2, 2.0 / 3.0)
    Dg = po.diagonal(Lf, model, Cs[1], bc.type)
    ref = po.fsmooth(Lf, model, Cs[1], bc.type, Dg, x, b, 2, 2.0 / 3.0)
    out = host(xd)
    assert normwise_err(out, ref) <= TOL64
    assert np.all(out[:, 0] == 0) and np.all(out[:, -1] == 0)  # the ring zeroed by Fsmooth


@pytest.mark.parametrize("model", MODELS)
def test_fsmooth_fp32_tiled(model, monkeypatch):
    monkeypatch.setenv("AE_TILED32", "1")
    rng, L, Cf, bc, op = make_case(model, 24, "pull_z", False, 91)
    x = rng.standard_normal((3,) + L.shape).astype(np.float32)
    b = rng.standard_normal((3,) + L.shape).astype(np.float32)
    xd = dev(x)
    op.Fsmooth(0, 0, Field(xd), Field(dev(b)), 2, 2.0 / 3.0)
    Dg = po.diagonal(L, model, Cf, bc.type)
    ref = po.fsmooth(L, model, Cf, bc.type, Dg, x.astype(np.float64), b.astype(np.float64), 2, 2.0 / 3.0)
    assert normwise_err(host(xd).astype(np.float64), ref) <= 1e-4
