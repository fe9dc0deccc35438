"""The GPU operator functions, through the C ABI, against the committed golden fixtures
(tests/golden/elastic_ops.npz): an 8 x 6 x 10-cell box with anisotropic spacing, random per-face
BC tables, all three stiffness kinds.  Same tolerances as the live-oracle parity tests: every node
within 1e-12 of the field's max-norm for FP64 arithmetic; restriction and interpolation within
1e-15."""
import os

import numpy as np
import pytest

from anisotropicfracture_gb300.elastic import BCElastic, Elastic, Field, level_desc
from helpers import golden_case, normwise_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "elastic_ops.npz")
TOL64 = 1e-12


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def operator(z, c, uniform):
    cells = tuple(int(v) for v in z["cells"])
    bc = BCElastic()
    bc.type[:] = c["bc_type"]
    bc.val[:] = c["bc_val"]
    op = Elastic([level_desc(cells)], int(c["model"]))
    op.SetModel(0, Field(c["C"]))
    op.SetBC(bc)
    op.SetUniform(uniform)
    op.prepareForSolve()
    return op


@pytest.mark.parametrize("name", ["iso", "mm", "diag"])
def test_operator_functions_match_golden(name):
    z = np.load(PATH)
    c = golden_case(z, name)
    shape = c["u"].shape
    op = operator(z, c, False)

    f = torch.zeros(shape, dtype=torch.float64, device="cuda")
    op.Fapply(0, 0, Field(f), Field(dev(c["u"])))
    assert normwise_err(host(f), c["fapply"]) <= TOL64

    dg = torch.zeros(shape, dtype=torch.float64, device="cuda")
    op.Diagonal(0, 0, Field(dg))
    assert normwise_err(host(dg), c["diag"]) <= TOL64

    xd = dev(c["x"])
    op.Fsmooth(0, 0, Field(xd), Field(dev(c["b"])), 2, 2.0 / 3.0)
    assert normwise_err(host(xd), c["fsmooth"]) <= TOL64

    r = torch.zeros(shape, dtype=torch.float64, device="cuda")
    nrm = op.Residual(0, 0, Field(r), Field(dev(c["x"])), Field(dev(c["b"])))
    assert normwise_err(host(r), c["resid"]) <= TOL64
    assert abs(nrm - float(c["resid_norm"])) <= TOL64 * float(c["resid_norm"])

    crse = torch.zeros(c["restrict"].shape, dtype=torch.float64, device="cuda")
    op.restriction(0, 1, Field(crse), Field(dev(c["u"])))
    assert normwise_err(host(crse), c["restrict"]) <= 1e-15
    fd = dev(c["x"])
    op.interpolation(0, 0, Field(fd), Field(dev(c["crse"])))
    assert normwise_err(host(fd), c["interp"]) <= 1e-15

    opu = operator(z, c, True)
    fu = torch.zeros(shape, dtype=torch.float64, device="cuda")
    opu.Fapply(0, 0, Field(fu), Field(dev(c["u"])))
    assert normwise_err(host(fu), c["fapply_uniform"]) <= TOL64
