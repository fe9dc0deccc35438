"""Composite solves over AMR levels made of several patches (separated boxes of one level, each
nested in one patch of the level below) on the GPU, against the oracle's composite restatement
(tests/test_oracle_multipatch.py pins it to the reference's multi-level known-answer tests):
FP64 iteration count within one and displacement within 1e-8, mixed precision within 1e-7 of a
tight FP64 oracle solution, the uniaxial known answer, and the solution independent of the order
the patches are listed in (bit for bit)."""
import numpy as np
import pytest

from anisotropicfracture_gb300 import microstructure, models
from anisotropicfracture_gb300.elastic import Elastic, Field, Linear
from helpers import bc_pull_z
from oracle import pyoracle as po
from test_gpu_amr import descs, lo_of
from test_oracle_multipatch import _uniaxial, _valid, patches

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def polycrystal(Ls, seed=5):
    seeds = microstructure.voronoi_seeds(12, seed)
    tab = models.cubic(1.68, 1.21, 0.75, models.random_rotations(12, np.random.default_rng(seed + 1)))
    Cs = []
    for L in Ls:
        lo = [L.lo[d] - L.ng for d in range(3)]
        hi = [L.hi[d] + L.ng for d in range(3)]
        g = microstructure.voronoi_grain_ids(lo, hi, tuple(L.dx), seeds)
        Cs.append(np.ascontiguousarray(np.moveaxis(tab[g], -1, 0)))
    bc = bc_pull_z()
    bs = [po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape)) for L in Ls]
    return Cs, bc, bs


def solve(Ls, model, Cs, bc, bs, precision="fp64", tol=1e-8, order=None):
    order = list(range(len(Ls))) if order is None else order
    Lo = [Ls[p] for p in order]
    op = Elastic(descs(Lo), model)
    for a, p in enumerate(order):
        op.SetModel(a, Field(Cs[p], lo_of(Ls[p])))
    op.SetBC(bc)
    op.SetUniform(False)
    s = Linear(op)
    s.setMaxFmgIter(0)
    s.setBottomSolver("cg")
    s.setPreSmooth(1)
    s.setPostSmooth(1)
    s.setPrecision(precision)
    xs = [np.zeros_like(bs[p]) for p in order]
    s.solve([Field(x, lo_of(Ls[p])) for x, p in zip(xs, order)], [Field(bs[p], lo_of(Ls[p])) for p in order],
            tol, 0.0)
    op.close()
    out = [None] * len(Ls)
    for x, p in zip(xs, order):
        out[p] = x
    return out, s.stats


@pytest.mark.parametrize("three", [False, True])
def test_multipatch_fp64_matches_oracle(three):
    Ls = patches(32, three)
    Cs, bc, bs = polycrystal(Ls)
    ref, st, rc = po.solve_amr(Ls, po.ORC_MAJORMINOR, Cs, bc.type, [np.zeros_like(b) for b in bs], bs, 1e-8, 0.0,
                               max_fmg_iter=0, bottom=0, nu1=1, nu2=1)
    assert rc == 0
    xs, stats = solve(Ls, models.MAJORMINOR, Cs, bc, bs)
    assert stats.converged and abs(stats.iters - st.iters) <= 1
    scale = max(np.abs(_valid(r, L)).max() for r, L in zip(ref, Ls))
    assert max(np.abs(_valid(x, L) - _valid(r, L)).max() for x, r, L in zip(xs, ref, Ls)) / scale < 1e-8


def test_multipatch_mixed_matches_oracle():
    Ls = patches(32, True)
    Cs, bc, bs = polycrystal(Ls)
    ref, st, rc = po.solve_amr(Ls, po.ORC_MAJORMINOR, Cs, bc.type, [np.zeros_like(b) for b in bs], bs, 1e-10, 0.0,
                               max_fmg_iter=0, bottom=0, nu1=1, nu2=1, max_iter=400)
    assert rc == 0
    xs, stats = solve(Ls, models.MAJORMINOR, Cs, bc, bs, precision="mixed")
    assert stats.converged and stats.resfinal <= stats.target
    scale = max(np.abs(_valid(r, L)).max() for r, L in zip(ref, Ls))
    assert max(np.abs(_valid(x, L) - _valid(r, L)).max() for x, r, L in zip(xs, ref, Ls)) / scale < 1e-7


def test_multipatch_uniaxial_known_answer():
    Ls = patches(32, True)
    bc, bs, _, Cs, ex = _uniaxial(Ls)
    xs, stats = solve(Ls, models.ISOTROPIC, Cs, bc, bs, tol=1e-10)
    assert stats.converged
    err = max(np.abs(_valid(x, L)[0] - _valid(e[None], L)[0]).max() for x, e, L in zip(xs, ex, Ls))
    assert err < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_patch_order_does_not_matter(precision):
    Ls = patches(32, True)
    Cs, bc, bs = polycrystal(Ls)
    x1, s1 = solve(Ls, models.MAJORMINOR, Cs, bc, bs, precision)
    x2, s2 = solve(Ls, models.MAJORMINOR, Cs, bc, bs, precision, order=[0, 2, 1, 4, 3])
    assert s1.iters == s2.iters
    for a, b in zip(x1, x2):
        assert np.array_equal(a, b)
