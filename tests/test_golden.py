"""The committed golden fixtures (tests/golden/elastic_ops.npz, written by
tests/golden/make_golden.py) against the oracle built on this machine.

The fixtures are the FP64 oracle's own outputs, so these tests pin the oracle across platforms and
changes: the operator functions use no library math and the oracle is built without contraction,
so they must agree to the last bit; the solve's Krylov dot products are summed in an order that
depends on the thread count, so it is held to its iteration count (+-1) and to 1e-9."""
import os

import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from helpers import golden_case, normwise_err
from oracle import pyoracle as po

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "elastic_ops.npz")
CASES = ["iso", "mm", "diag"]


@pytest.fixture(scope="module")
def z():
    return np.load(PATH)


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_operator_fixtures(z, name):
    c = golden_case(z, name)
    model, C, bt = int(c["model"]), c["C"], c["bc_type"]
    L = po.level(tuple(int(v) for v in z["cells"]))
    assert C.shape[1:] == L.shape
    assert np.array_equal(po.fapply(L, model, C, bt, c["u"]), c["fapply"])
    assert np.array_equal(po.fapply(L, model, C, bt, c["u"], True), c["fapply_uniform"])
    dg = po.diagonal(L, model, C, bt)
    assert np.array_equal(dg, c["diag"])
    assert np.array_equal(po.fsmooth(L, model, C, bt, dg, c["x"], c["b"], 2, 2.0 / 3.0), c["fsmooth"])
    r, rn = po.residual(L, model, C, bt, c["x"], c["b"])
    assert np.array_equal(r, c["resid"]) and rn == float(c["resid_norm"])
    Lc = po.coarsen(L)
    assert np.array_equal(po.restrict(Lc, L, c["u"]), c["restrict"])
    assert np.array_equal(po.interp_add(L, Lc, c["x"], c["crse"]), c["interp"])


def test_fixture_inputs_are_exact_in_fp32(z):
    """Inputs are multiples of 1/64, so an FP32 kernel reads exactly the FP64 inputs."""
    for name in CASES:
        c = golden_case(z, name)
        for k in ("u", "x", "b", "crse"):
            assert np.array_equal(c[k].astype(np.float32).astype(np.float64), c[k])


def test_oracle_reproduces_solve_fixture(z):
    c = golden_case(z, "solve")
    L = po.level(tuple(int(v) for v in z["solve_cells"]))
    b = po.bc_init(L, c["bc_type"], c["bc_val"], np.zeros((3,) + L.shape))
    assert np.array_equal(b, c["b"])
    u, st, rc = po.solve(L, models.MAJORMINOR, c["C"], c["bc_type"], np.zeros_like(b), b, 1e-8, 0.0)
    assert rc == 0 and st.converged
    assert abs(st.iters - int(c["iters"])) <= 1
    assert normwise_err(u, c["u"]) < 1e-9
