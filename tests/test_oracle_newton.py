"""Pins the oracle's Newton<T> pieces (CPU only): the Newton right-hand side b - N(u) of
src/Solver/Nonlocal/Newton.H:30-139 and the DW / W fields of Newton.H:233-333, for the linear
and affine models (DW = C : (grad u - F0))."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from helpers import bc_random, normwise_err, random_coeffs
from oracle import pyoracle as po

MM, ISO = po.ORC_MAJORMINOR, po.ORC_ISOTROPIC


def _uniform(model, shape, rng):
    c = random_coeffs(model, (1, 1, 1), rng)[:, 0, 0, 0]
    return np.ascontiguousarray(np.broadcast_to(c[:, None, None, None], (c.size,) + shape))


def test_newton_rhs_of_zero_displacement_is_b():
    rng = np.random.default_rng(1)
    L = po.level((8, 7, 6))
    Cf = random_coeffs(MM, L.shape, rng)
    b = rng.standard_normal((3,) + L.shape)
    rhs = po.newton_residual(L, MM, Cf, bc_random(rng).type, np.zeros_like(b), b)
    assert np.array_equal(rhs, b)


@pytest.mark.parametrize("model", [MM, ISO])
def test_newton_rhs_inside_is_b_minus_A_u_on_quadratics(model):
    """Central differences are exact on quadratics, so two nodes away from the boundary the wide
    div(C : grad u) equals the compact operator; uniform stiffness."""
    rng = np.random.default_rng(2)
    L = po.level(10)
    Cf = _uniform(model, L.shape, rng)
    X, Y, Z = po.node_coords(L)
    u = np.stack([0.3 * X * X + 0.1 * X * Y - 0.2 * Z, 0.2 * Y * Z + 0.05 * X, 0.4 * Z * Z - 0.3 * X * Z])
    u = np.ascontiguousarray(u)
    b = rng.standard_normal((3,) + L.shape)
    bct = np.zeros((26, 3), np.int32)
    rhs = po.newton_residual(L, model, Cf, bct, u, b)
    Au = po.fapply(L, model, Cf, bct, u, uniform=True)
    inner = (slice(None), slice(2, -2), slice(2, -2), slice(2, -2))
    assert normwise_err(rhs[inner], (b - Au)[inner]) < 1e-10


def test_affine_eigenstrain_enters_through_traction_rows():
    """u = 0 with a uniform eigenstrain F0: inside, div(C : (-F0)) = 0; on a traction face the row
    is sigma n with sigma = -C : F0, so rhs = b + (C : F0) n there."""
    rng = np.random.default_rng(3)
    L = po.level(6)
    Cf = _uniform(ISO, L.shape, rng)
    F0v = 0.01 * rng.standard_normal((3, 3))
    F0 = np.ascontiguousarray(np.broadcast_to(F0v.reshape(9, 1, 1, 1), (9,) + L.shape))
    bct = np.full((26, 3), 1, np.int32)  # traction everywhere
    b = np.zeros((3,) + L.shape)
    rhs = po.newton_residual(L, ISO, Cf, bct, np.zeros_like(b), b, F0=F0)
    lam, mu = Cf[0, 0, 0, 0], Cf[1, 0, 0, 0]
    sig = lam * np.trace(F0v) * np.eye(3) + mu * (F0v + F0v.T)
    # the x-lo face (interior of the face): normal (-1, 0, 0)
    assert np.allclose(rhs[:, 3, 3, 0], sig @ np.array([-1.0, 0, 0]), rtol=1e-12, atol=1e-15)
    assert np.allclose(rhs[:, 2:-2, 2:-2, 2:-2], 0.0, atol=1e-15)


def test_newton_dw_and_w():
    rng = np.random.default_rng(4)
    L = po.level((7, 6, 5))
    u = rng.standard_normal((3,) + L.shape)
    for model in (MM, ISO):
        Cf = random_coeffs(model, L.shape, rng)
        dw, w = po.newton_dw(L, model, Cf, u)
        sig = po.stress(L, model, Cf, u, voigt=False)  # Elastic<T>::Stress, same stencils
        assert normwise_err(dw, sig) < 1e-14
        g = dw.reshape((3, 3) + L.shape)
        # W = 0.5 grad u : sigma for the linear models (sigma is symmetric: grad u : sigma = eps : sigma)
        strain = po.strain(L, u, voigt=False).reshape((3, 3) + L.shape)
        Ww = 0.5 * (strain * g).sum(axis=(0, 1))
        assert normwise_err(w, Ww) < 1e-13
        F0 = 0.01 * rng.standard_normal((9,) + L.shape)
        dwa, wa = po.newton_dw(L, model, Cf, u, F0=F0)
        dw0, _ = po.newton_dw(L, model, Cf, np.zeros_like(u), F0=F0)
        assert normwise_err(dwa, dw + dw0) < 1e-12  # DW is affine in grad u - F0
