"""The stencil-free first sweep of a smoother call that starts from a zero correction (the
pre-smoothing of every V-cycle level, each patch's mini-cycle) against the full sweep over the
zero-filled correction (AE_ZERO_SWEEP=0, read when an operator is created).  A 0 is zero on every
row, so the two must give the same solves bit for bit (tolerance 0): FP64 and mixed precision, one
level and two AMR levels, per-node stiffness and a grain map, CG and BiCGStab bottoms."""
import os

import numpy as np
import pytest

from anisotropicfracture_gb300 import microstructure, models
from anisotropicfracture_gb300.elastic import Elastic, Field, Linear
from helpers import polycrystal_amr
from test_gpu_amr import descs, lo_of

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _solve(zero, Ls, Cs, bc, bs, precision, grains, bottom):
    os.environ["AE_ZERO_SWEEP"] = "1" if zero else "0"
    try:
        op = Elastic(descs(Ls), models.MAJORMINOR)
    finally:
        os.environ.pop("AE_ZERO_SWEEP", None)
    for a, L in enumerate(Ls):
        if grains:
            seeds = microstructure.voronoi_seeds(12, 9)
            tab = models.cubic(1.68, 1.21, 0.75, models.random_rotations(12, np.random.default_rng(10)))
            lo = [L.lo[d] - L.ng for d in range(3)]
            hi = [L.hi[d] + L.ng for d in range(3)]
            g = microstructure.voronoi_grain_ids(lo, hi, tuple(L.dx), seeds).astype(np.int32)
            op.SetModelGrains(a, Field(np.ascontiguousarray(g[None]), lo_of(L)), tab)
        else:
            op.SetModel(a, Field(Cs[a], lo_of(L)))
    op.SetBC(bc)
    op.SetUniform(False)
    s = Linear(op)
    s.setMaxFmgIter(0)
    s.setBottomSolver(bottom)
    s.setPreSmooth(2)
    s.setPostSmooth(2)
    s.setPrecision(precision)
    xs = [np.zeros_like(b) for b in bs]
    s.solve([Field(x, lo_of(L)) for x, L in zip(xs, Ls)], [Field(b, lo_of(L)) for b, L in zip(bs, Ls)], 1e-8, 0.0)
    st = s.stats
    op.close()
    return xs, st.iters


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nlev", [1, 2])
@pytest.mark.parametrize("grains", [False, True])
def test_zero_start_sweep_is_the_full_sweep(precision, nlev, grains):
    Ls, Cs, bc, bs = polycrystal_amr(24, nlev)
    ref, it_ref = _solve(False, Ls, Cs, bc, bs, precision, grains, "cg")
    got, it_got = _solve(True, Ls, Cs, bc, bs, precision, grains, "cg")
    assert it_got == it_ref
    for a, b in zip(got, ref):
        assert np.array_equal(a, b), float(np.abs(a - b).max())


def test_zero_start_sweep_with_bicgstab_bottom():
    Ls, Cs, bc, bs = polycrystal_amr(24, 2)
    ref, _ = _solve(False, Ls, Cs, bc, bs, "mixed", True, "bicgstab")
    got, _ = _solve(True, Ls, Cs, bc, bs, "mixed", True, "bicgstab")
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
