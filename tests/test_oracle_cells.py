"""Pins the oracle's periodic-cell restatement (CPU only).

The periodic operator is the reference's interior row with neighbours taken modulo the cell.  It
is pinned three ways: against the already-pinned box oracle on a box padded with periodic images
(so every periodic node is an interior node there), against the exact discrete Fourier symbol of
the stencils for a uniform stiffness, and against closed-form homogenisation results (a uniform
cell carries no fluctuation; a laminate's normal stress tends to the harmonic (Reuss) mean)."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import cells, models
from helpers import normwise_err, random_coeffs
from oracle import pyoracle as po

MODELS = [models.ISOTROPIC, models.MAJORMINOR, models.DIAGONAL]


def _pad(a, g=2):
    """Periodic images: a box of nodes -g .. n-1+g around the cell (last three axes)."""
    return np.ascontiguousarray(np.pad(a, [(0, 0)] + [(g, g)] * 3, mode="wrap"))


def _box_for(n, g=2):
    """A non-periodic level whose nodes 0 .. n-1+2g hold the padded cell, same spacing."""
    n = (n,) * 3 if np.isscalar(n) else tuple(n)
    return po.level(tuple(c + 2 * g - 1 for c in n), dx=tuple(1.0 / c for c in n))


def _inner(a, g=2):
    return a[..., g:-g, g:-g, g:-g]


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("uniform", [False, True])
def test_cell_fapply_is_the_interior_row_on_periodic_images(model, uniform):
    rng = np.random.default_rng(11 + model)
    n = (6, 5, 4)
    L = po.rve_level(n)
    Cf = random_coeffs(model, L.shape, rng)
    u = rng.standard_normal((3,) + L.shape)
    f = po.rve_fapply(L, model, Cf, u, uniform=uniform)
    Lb = _box_for(n)
    fb = po.fapply(Lb, model, _pad(Cf), np.zeros((26, 3), np.int32), _pad(u), uniform=uniform)
    assert normwise_err(f, _inner(fb)) < 1e-13


@pytest.mark.parametrize("model", MODELS)
def test_cell_diagonal_is_the_interior_diagonal(model):
    rng = np.random.default_rng(5)
    n = (4, 6, 5)
    L = po.rve_level(n)
    Cf = random_coeffs(model, L.shape, rng)
    D = po.rve_diagonal(L, model, Cf)
    Db = po.diagonal(_box_for(n), model, _pad(Cf), np.zeros((26, 3), np.int32))
    assert normwise_err(D, _inner(Db)) < 1e-14


def test_cell_fapply_fourier_symbol():
    """u = a cos(2 pi k.x + phi) under a uniform stiffness: the stencils act exactly as
    D_jj -> -4 sin^2(theta_j / 2) / h_j^2 and D_jl -> -sin(theta_j) sin(theta_l) / (h_j h_l),
    theta_j = 2 pi k_j h_j, so f_i = -C_ijkl a_k M_jl cos(.)."""
    n = (8, 6, 10)
    L = po.rve_level(n)
    R = models.random_rotations(1, np.random.default_rng(3))
    c21 = models.cubic(1.68, 1.21, 0.75, R)[0]
    Cfull = models.full_from_slots(c21)
    Cf = np.ascontiguousarray(np.broadcast_to(c21[:, None, None, None], (21,) + L.shape))
    kv = np.array([1, 2, 3])
    h = np.array([1.0 / c for c in n])
    a = np.array([0.3, -0.7, 0.2])
    z, y, x = np.meshgrid(*[np.arange(c) * hh for c, hh in zip(n[::-1], h[::-1])], indexing="ij")
    ph = 2 * np.pi * (kv[0] * x + kv[1] * y + kv[2] * z) + 0.4
    u = np.ascontiguousarray(a[:, None, None, None] * np.cos(ph)[None])
    f = po.rve_fapply(L, models.MAJORMINOR, Cf, u, uniform=True)
    th = 2 * np.pi * kv * h
    M = np.outer(np.sin(th), np.sin(th)) / np.outer(h, h)
    for j in range(3):
        M[j, j] = 4 * np.sin(th[j] / 2) ** 2 / h[j] ** 2
    amp = -np.einsum("ijkl,k,jl->i", Cfull, a, M)
    ex = amp[:, None, None, None] * np.cos(ph)[None]
    assert normwise_err(f, ex) < 1e-12


@pytest.mark.parametrize("model", MODELS)
def test_cell_rhs_is_minus_A_of_the_affine_field(model):
    """A(E x) = sum_d (d_d C) : E e_d exactly (the stencils are exact on affine fields), so the
    box oracle applied to E x on the padded images (a non-periodic affine field) gives -b."""
    rng = np.random.default_rng(9)
    n = (5, 6, 4)
    L = po.rve_level(n)
    Cf = random_coeffs(model, L.shape, rng)
    E = rng.standard_normal((3, 3)) * 1e-3
    b = po.rve_rhs(L, model, Cf, E)
    Lb = _box_for(n)
    X, Y, Z = po.node_coords(Lb)
    xs = np.stack([X, Y, Z])
    u = np.ascontiguousarray(np.einsum("kl,lzyx->kzyx", E, xs))
    fb = po.fapply(Lb, model, _pad(Cf), np.zeros((26, 3), np.int32), u)
    assert normwise_err(b, -_inner(fb)) < 1e-12
    assert np.abs(b.sum(axis=(1, 2, 3))).max() < 1e-12 * np.abs(b).sum()  # telescoping sum


def test_cell_transfers_match_the_interior_weights():
    rng = np.random.default_rng(2)
    nf = (8, 6, 4)
    Lf, Lc = po.rve_level(nf), po.rve_coarsen(po.rve_level(nf))
    fine = rng.standard_normal((3,) + Lf.shape)
    crse = po.rve_restrict(Lc, Lf, fine)
    # the box oracle's interior weights on padded images: coarse node I sits at fine 2I
    Lbf = _box_for(nf)
    Lbc = po.coarsen(Lbf)
    cb = np.zeros((3,) + Lbc.shape)
    cb = po.restrict(Lbc, Lbf, _pad(fine))
    assert normwise_err(crse, cb[:, 1:-1, 1:-1, 1:-1]) < 1e-14
    # constants are restricted and interpolated exactly; interpolation keeps coarse values
    one = np.ones((1,) + Lf.shape)
    assert np.allclose(po.rve_restrict(Lc, Lf, one), 1.0, atol=1e-15)
    c = rng.standard_normal((2,) + Lc.shape)
    fi = po.rve_interp_add(Lf, Lc, np.zeros((2,) + Lf.shape), c)
    assert np.array_equal(fi[:, ::2, ::2, ::2], c)
    fb = po.interp_add(Lbf, Lbc, np.zeros((2,) + Lbf.shape), _pad(c, 1))
    assert normwise_err(fi, _inner(fb)) < 1e-14


def test_uniform_cell_has_no_fluctuation():
    n = 8
    L = po.rve_level(n)
    c21 = models.cubic(1.68, 1.21, 0.75, models.random_rotations(1, np.random.default_rng(1)))[0]
    Cf = np.ascontiguousarray(np.broadcast_to(c21[:, None, None, None], (21,) + L.shape))
    E = cells.unit_strains()[3]
    w, st, rc, bf = po.rve_solve(L, models.MAJORMINOR, Cf, E)
    assert rc == 0 and np.abs(w).max() == 0.0
    sig = po.rve_mean_stress(L, models.MAJORMINOR, Cf, E, w)
    ref = np.einsum("ijkl,kl->ij", models.full_from_slots(c21), E)
    assert np.abs(sig - ref).max() <= 1e-14 * np.abs(ref).max()


def test_laminate_normal_stress_tends_to_the_reuss_mean():
    """Isotropic layers varying smoothly along x under E = e_x e_x: the exact cell solution has a
    uniform sigma_xx = E_xx / mean(1 / (lambda + 2 mu)).  Second-order stencils: 0.1 % at 32 cells."""
    n = 32
    L = po.rve_level(n)
    x = np.arange(n) / n
    mu = 1.0 + 0.5 * np.sin(2 * np.pi * x)
    lam = 1.5 + 0.5 * np.cos(2 * np.pi * x)
    Cf = np.zeros((2,) + L.shape)
    Cf[0] = lam[None, None, :]
    Cf[1] = mu[None, None, :]
    E = np.zeros((3, 3))
    E[0, 0] = 1e-3
    w, st, rc, bf = po.rve_solve(L, models.ISOTROPIC, Cf, E, bottom=1, nu1=2, nu2=2)
    assert rc == 0
    sig = po.rve_mean_stress(L, models.ISOTROPIC, Cf, E, w)
    xs = np.linspace(0, 1, 20001)[:-1]
    reuss = 1e-3 / np.mean(1.0 / (1.5 + 0.5 * np.cos(2 * np.pi * xs) + 2 * (1.0 + 0.5 * np.sin(2 * np.pi * xs))))
    assert abs(sig[0, 0] - reuss) < 1e-3 * reuss
    assert abs(w.mean()) < 1e-15


def test_cell_solve_residual_and_body_force():
    """The converged cell solve meets its own test on an independent evaluation of b - A w, the
    mean of which is the body force it reports; w has zero mean."""
    n = 16
    L = po.rve_level(n)
    seeds, table = cells.rve_grains(n, 8, seed=5)
    Cf = cells.rve_stiffness(n, seeds, table)
    E = cells.unit_strains()[0]
    w, st, rc, bf = po.rve_solve(L, models.MAJORMINOR, Cf, E, bottom=1, nu1=2, nu2=2, tol_rel=1e-8)
    assert rc == 0 and st.converged
    b = po.rve_rhs(L, models.MAJORMINOR, Cf, E)
    r, mean, nrm = po.rve_residual(L, models.MAJORMINOR, Cf, w, b)
    assert nrm <= st.target * (1 + 1e-12)
    assert np.allclose(mean, bf, rtol=1e-10, atol=1e-20)
    assert np.abs(w.mean(axis=(1, 2, 3))).max() < 1e-16
    # the multiplier is small against the load (the discretisation's lack of conservation)
    assert np.abs(bf).max() < 1e-2 * np.abs(b).max()


def test_oracle_cell_levels():
    assert po.rve_num_mg_levels(po.rve_level(16)) == 4   # 16 8 4 2
    assert po.rve_num_mg_levels(po.rve_level(24)) == 4   # 24 12 6 3
    assert po.rve_num_mg_levels(po.rve_level(40)) == 4   # 40 20 10 5
    assert po.rve_num_mg_levels(po.rve_level(7)) == 1
