"""The CUDA path, through the C ABI, against outputs of the REFERENCE'S OWN CODE
(tests/golden/ref_ops.npz; see tests/golden/make_ref_golden.py): Fapply (with and without
m_uniform), Diagonal, Fsmooth, Strain / Stress / Energy, restriction, interpolation, BC Init and
the coarse-level stiffness of averageDownCoeffsSameAmrLevel, for the isotropic, MajorMinor,
Diagonal and Sym::Major (NeoHookean tangent; no Stress / Energy) kinds, on an 8 x 6 x 10-cell level with
anisotropic spacing and a random BC table; Fapply / Diagonal / Fsmooth also on two refined
patches with ghost layers (one inside the domain, one touching two domain faces), run as AMR
level 1 of a two-level operator.

Tolerance (FP64), both required: every node within 1e-12 of the field's max-norm, and
|gpu - ref| <= 1e-12 * max(|ref_node|, 1e-3 * max|ref|) per node (helpers.pernode_err).  The
kernels fuse multiply-adds that the reference rounds separately.  Transfers and BC Init involve
no fused products and must be bitwise."""
import os

import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300.elastic import BCElastic, Elastic, Field, level_desc
from helpers import golden_level, golden_prefixed, normwise_err, pernode_err
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ops.npz")
NAMES = {"iso": models.ISOTROPIC, "mm": models.MAJORMINOR, "diag": models.DIAGONAL, "major": models.MAJOR}
TOL64 = 1e-12


@pytest.fixture(scope="module")
def z():
    return np.load(PATH)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def close(got, ref, what):
    assert normwise_err(got, ref) <= TOL64, what
    assert pernode_err(got, ref) <= TOL64, what


def bc_of(c):
    bc = BCElastic()
    bc.type[:] = c["bc_type"]
    bc.val[:] = c["bc_val"]
    return bc


def box_operator(z, c, uniform):
    cells = tuple(int(v) for v in z["cells"])
    op = Elastic([level_desc(cells, dx=tuple(float(v) for v in z["dx"]))], int(c["model"]))
    op.SetModel(0, Field(c["C"]))
    op.SetBC(bc_of(c))
    op.SetUniform(uniform)
    op.prepareForSolve()
    return op


@pytest.mark.parametrize("name", list(NAMES))
def test_box_operator_matches_reference_code(z, name):
    c = golden_prefixed(z, "box_%s_" % name)
    shape = c["u"].shape
    op = box_operator(z, c, False)
    f = torch.zeros(shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(c["u"])))
    close(host(f), c["fapply"], "Fapply")
    dg = torch.zeros(shape, dtype=torch.float64, device="cuda")
    op.Diagonal(0, 0, Field(dg))
    close(host(dg), c["diag"], "Diagonal")
    xd = dev(c["x"])
    op.Fsmooth(0, 0, Field(xd), Field(dev(c["b"])), 2, 2.0 / 3.0)
    close(host(xd), c["fsmooth"], "Fsmooth")
    if name != "major":  # Stress / Energy evaluate a linear model
        _stress_energy(op, c, shape)
    # the stiffness the reference coarsens onto the next multigrid level drives the GPU's
    # coarse-level operator: its Fapply equals the oracle's Fapply with the reference's coarse C
    Lc = po.coarsen(golden_level(z, "box"))
    uc = np.random.default_rng(5).standard_normal((3,) + Lc.shape)
    fc = torch.zeros((3,) + Lc.shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 1, Field(fc), Field(dev(uc)))
    close(host(fc), po.fapply(Lc, NAMES[name], c["coarse_C"], c["bc_type"], uc), "coarse-level Fapply")
    opu = box_operator(z, c, True)
    fu = torch.zeros(shape, dtype=torch.float64, device="cuda")
    opu.Fapply(0, 0, Field(fu), Field(dev(c["u"])))
    close(host(fu), c["fapply_uniform"], "Fapply m_uniform")


def _stress_energy(op, c, shape):
    sig = torch.zeros((9,) + shape[1:], dtype=torch.float64, device="cuda")
    op.Stress(0, Field(sig), Field(dev(c["u"])))
    close(host(sig), c["stress"], "Stress")
    sv = torch.zeros((6,) + shape[1:], dtype=torch.float64, device="cuda")
    op.Stress(0, Field(sv), Field(dev(c["u"])), voigt=True)
    close(host(sv), c["stress_voigt"], "Stress voigt")
    w = torch.zeros((1,) + shape[1:], dtype=torch.float64, device="cuda")
    op.Energy(0, Field(w), Field(dev(c["u"])))
    close(host(w), c["energy"], "Energy")


def test_fields_and_transfers_match_reference_code(z):
    c = golden_prefixed(z, "fields_")
    cells = tuple(int(v) for v in z["cells"])
    shape = c["u"].shape
    op = Elastic([level_desc(cells, dx=tuple(float(v) for v in z["dx"]))], models.ISOTROPIC)
    op.SetModel(0, Field(np.ones((2,) + shape[1:])))
    bc = BCElastic()
    bc.type[:] = c["bc_type"]
    bc.val[:] = c["bc_val"]
    op.SetBC(bc)
    op.prepareForSolve()
    eps = torch.zeros((9,) + shape[1:], dtype=torch.float64, device="cuda")
    op.Strain(0, Field(eps), Field(dev(c["u"])))
    close(host(eps), c["strain"], "Strain")
    ev = torch.zeros((6,) + shape[1:], dtype=torch.float64, device="cuda")
    op.Strain(0, Field(ev), Field(dev(c["u"])), voigt=True)
    close(host(ev), c["strain_voigt"], "Strain voigt")
    crse = torch.zeros(c["crse"].shape, dtype=torch.float64, device="cuda")
    op.restriction(0, 1, Field(crse), Field(dev(c["u"])))
    assert np.array_equal(host(crse), c["restrict"])
    fd = dev(c["x"])
    op.interpolation(0, 0, Field(fd), Field(dev(c["crse"])))
    assert np.array_equal(host(fd), c["interp"])
    for homog, key in ((False, "bc_init"), (True, "bc_init_homog")):
        r = dev(c["r0"])
        op.BCInit(0, Field(r), homogeneous=homog)
        assert np.array_equal(host(r), c[key]), key


@pytest.mark.parametrize("lname", ["patch", "edge"])
@pytest.mark.parametrize("name", list(NAMES))
def test_refined_patch_matches_reference_code(z, lname, name):
    L = golden_level(z, lname)
    c = golden_prefixed(z, "%s_%s_" % (lname, name))
    model = NAMES[name]
    n = L.dom_hi[0] - L.dom_lo[0]
    lo = tuple(L.lo[d] for d in range(3))
    hi = tuple(L.hi[d] for d in range(3))
    store_lo = tuple(L.lo[d] - L.ng for d in range(3))
    op = Elastic([level_desc(n // 2), level_desc(n, lo=lo, hi=hi)], model)
    coarse_shape = (n // 2 + 1,) * 3
    op.SetModel(0, Field(np.ascontiguousarray(np.broadcast_to(c["C"][:, :1, :1, :1],
                                                              (c["C"].shape[0],) + coarse_shape))))
    op.SetModel(1, Field(c["C"], store_lo))
    op.SetBC(bc_of(c))
    op.SetUniform(False)
    op.prepareForSolve()
    shape = c["u"].shape
    f = torch.zeros(shape, dtype=torch.float64, device="cuda")
    op.Fapply(1, 0, Field(f, store_lo), Field(dev(c["u"]), store_lo))
    close(host(f), c["fapply"], "Fapply")
    dg = torch.zeros(shape, dtype=torch.float64, device="cuda")
    op.Diagonal(1, 0, Field(dg, store_lo))
    close(host(dg), c["diag"], "Diagonal")
    xd = dev(c["x"])
    op.Fsmooth(1, 0, Field(xd, store_lo), Field(dev(c["b"]), store_lo), 2, 2.0 / 3.0)
    close(host(xd), c["fsmooth"], "Fsmooth")
