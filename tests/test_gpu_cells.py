"""Batched periodic cells on the GPU (ae_batch_*), against the oracle's cell solve.

Tolerances: the FP64 batch runs the oracle's algorithm (same cycle, same bottom solver) in a
different summation order, so iteration counts agree and the solutions agree to 1e-9 of their
max-norm (rounding amplified by the iteration); cell-averaged stresses to 1e-9.  Mixed precision
reaches the same 1e-8 residual with a displacement error <= 1e-7 (relative max-norm) against the
FP64 result.  A solve's result does not depend on what else is in the batch, nor on the launch
shapes, bit for bit."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, cells, models
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MM = models.MAJORMINOR
OPTS = dict(max_fmg_iter=0, nu1=2, nu2=2, sweeps=2, bottom=1, bottom_max_iter=200, bottom_reltol=1e-4, nuf=8,
            max_iter=100)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _cell(n, ngr, seed):
    seeds, table = cells.rve_grains(n, ngr, seed)
    return seeds, table, cells.rve_stiffness(n, seeds, table)


def _batch(specs, loads, model=MM, grains=True):
    """specs: list of (n, ngrains, seed); loads: list per cell of 3x3 gradients."""
    B = cells.CellBatch([(n, len(L)) for (n, _, _), L in zip(specs, loads)], model)
    s = 0
    Cs = []
    for c, ((n, ngr, seed), L) in enumerate(zip(specs, loads)):
        seeds, table, Cf = _cell(n, ngr, seed)
        Cs.append(Cf)
        if grains:
            B.set_grains(c, seeds, table)
        else:
            B.set_model(c, Cf)
        for E in L:
            B.set_load(s, E)
            s += 1
    B.prepare()
    return B, Cs


@pytest.mark.parametrize("precision", [0, 1])
def test_device_voronoi_matches_host_voronoi(precision):
    """A Voronoi cell built on the device (grain ids + tables, read by the finest-level kernels)
    solves bit for bit like the same cell given as the host-built per-node field."""
    n = 12
    seeds, table, Cf = _cell(n, 9, seed=3)
    B = cells.CellBatch([(n, 1)])
    B.set_grains(0, seeds, table)
    B.set_load(0, cells.unit_strains()[0] + cells.unit_strains()[4])
    B.prepare()
    B2 = cells.CellBatch([(n, 1)])
    B2.set_model(0, Cf)
    B2.set_load(0, cells.unit_strains()[0] + cells.unit_strains()[4])
    B2.prepare()
    s1, _ = B.solve(precision=precision, inner_cycles=2, **OPTS)
    s2, _ = B2.solve(precision=precision, inner_cycles=2, **OPTS)
    assert s1[0]["iters"] == s2[0]["iters"]
    assert np.array_equal(B.solution(0), B2.solution(0))
    assert np.array_equal(s1[0]["mean_stress"], s2[0]["mean_stress"])


@pytest.mark.parametrize("n,ngr", [(16, 8), (12, 5), (10, 6)])
def test_fp64_batch_matches_oracle(n, ngr):
    E = cells.unit_strains()[0] + cells.unit_strains()[5]
    B, Cs = _batch([(n, ngr, 7)], [[E]])
    st, rc = B.solve(precision=0, **OPTS)
    w = B.solution(0)
    L = po.rve_level(n)
    wo, so, rco, bfo = po.rve_solve(L, MM, Cs[0], E, **OPTS)
    assert rc == 0 and rco == 0
    assert st[0]["iters"] == so.iters
    assert st[0]["nlevels"] == so.nlevels
    assert _rel(w, wo) < 1e-9
    sig_o = po.rve_mean_stress(L, MM, Cs[0], E, wo)
    assert _rel(st[0]["mean_stress"], sig_o) < 1e-9
    assert np.allclose(st[0]["body_force"], bfo, rtol=1e-3, atol=1e-14)


def test_mixed_precision_meets_the_fp64_result():
    E = cells.unit_strains()[3]
    specs = [(16, 8, 1), (24, 12, 2), (32, 16, 3)]
    B, Cs = _batch(specs, [[E]] * 3)
    s64, rc64 = B.solve(precision=0, **OPTS)
    w64 = [B.solution(s) for s in range(3)]
    s32, rc32 = B.solve(precision=1, inner_cycles=2, **OPTS)
    assert rc64 == 0 and rc32 == 0
    for s in range(3):
        assert s32[s]["converged"] and s32[s]["resfinal"] <= s32[s]["target"]
        assert _rel(B.solution(s), w64[s]) <= 1e-7


@pytest.mark.parametrize("precision", [0, 1])
def test_each_result_is_the_same_alone_and_in_the_mix(precision):
    Es = cells.unit_strains()
    specs = [(16, 8, 11), (24, 10, 12), (8, 4, 13), (32, 9, 14), (20, 7, 15)]
    loads = [[Es[0], Es[4]], [Es[1]], [Es[2], Es[3], Es[5]], [Es[0]], [Es[5]]]
    B, _ = _batch(specs, loads)
    st, rc = B.solve(precision=precision, inner_cycles=2, **OPTS)
    assert rc == 0
    mix = [B.solution(s) for s in range(B.nsolves)]
    s = 0
    for c, (spec, L) in enumerate(zip(specs, loads)):
        for k, E in enumerate(L):
            A, _ = _batch([spec], [[E]])
            sa, rca = A.solve(precision=precision, inner_cycles=2, **OPTS)
            assert rca == 0
            assert np.array_equal(A.solution(0), mix[s]), (c, k)
            assert sa[0]["iters"] == st[s]["iters"]
            assert np.array_equal(sa[0]["mean_stress"], st[s]["mean_stress"])
            s += 1


def test_launch_shapes_do_not_change_results():
    E = cells.unit_strains()[1]
    specs = [(16, 8, 21), (24, 8, 22)]
    B, _ = _batch(specs, [[E], [E]])
    B.solve(precision=1, inner_cycles=2, **OPTS)
    ref = [B.solution(s) for s in range(2)]
    for lev in range(4):
        B.set_shape(lev, 128, 7)
    B.solve(precision=1, inner_cycles=2, **OPTS)
    for s in range(2):
        assert np.array_equal(B.solution(s), ref[s])
    assert B.get_shape(0) == (128, 7)


def test_single_level_cell_and_fp32_inner_cycles():
    """An odd cell has one multigrid level: the solve is bottom solves only."""
    E = cells.unit_strains()[2]
    B, Cs = _batch([(7, 4, 31)], [[E]])
    assert B.num_levels(0) == 1
    st, rc = B.solve(precision=0, **OPTS)
    wo, so, rco, _ = po.rve_solve(po.rve_level(7), MM, Cs[0], E, **OPTS)
    assert rc == 0 and rco == 0 and st[0]["iters"] == so.iters
    assert _rel(B.solution(0), wo) < 1e-9


def _smooth_cell_coeffs(model, n, rng):
    """Smoothly varying periodic coefficients (damped Jacobi needs no sharp jumps here)."""
    x = np.arange(n) / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    nc = models.NCOEF[model]
    out = np.empty((nc, n, n, n))
    for q in range(nc):
        ph = rng.random(3) * 2 * np.pi
        base = (1.0 + rng.random()) if model == models.ISOTROPIC else (0.8 + 0.4 * rng.random())
        out[q] = base * (1.0 + 0.2 * np.sin(2 * np.pi * X + ph[0]) * np.cos(2 * np.pi * Y + ph[1])
                         + 0.1 * np.sin(2 * np.pi * Z + ph[2]))
    return np.ascontiguousarray(out)


def test_isotropic_and_diagonal_cells():
    rng = np.random.default_rng(4)
    for model in (models.ISOTROPIC, models.DIAGONAL):
        n = 12
        Cf = _smooth_cell_coeffs(model, n, rng)
        E = cells.unit_strains()[0]
        B = cells.CellBatch([(n, 1)], model)
        B.set_model(0, Cf)
        B.set_load(0, E)
        B.prepare()
        st, rc = B.solve(precision=0, **OPTS)
        wo, so, rco, _ = po.rve_solve(po.rve_level(n), model, Cf, E, **OPTS)
        assert rc == 0 and rco == 0
        assert st[0]["iters"] == so.iters
        assert _rel(B.solution(0), wo) < 1e-9


def test_nan_stiffness_is_rejected():
    n = 8
    _, _, Cf = _cell(n, 3, 1)
    Cf = Cf.copy()
    Cf[0, 2, 3, 4] = np.nan
    B = cells.CellBatch([(n, 1)])
    B.set_model(0, Cf)
    with pytest.raises(_lib.AeError) as e:
        B.prepare()
    assert e.value.code == _lib.AE_ERR_NAN


def test_bad_descriptors_are_rejected():
    lib = _lib.load()
    import ctypes as C
    h = C.c_void_p()
    d = cells.cell_desc(1, 1)
    assert lib.ae_batch_create(C.byref(d), 1, MM, C.byref(h)) == _lib.AE_ERR_ARG
    d = cells.cell_desc(8, 0)
    assert lib.ae_batch_create(C.byref(d), 1, MM, C.byref(h)) == _lib.AE_ERR_ARG
