"""ae_op_set_model_grains: a Voronoi stiffness given as grain ids and a per-grain table.

The sweeps then read 2-byte ids and the table instead of the per-node coefficients.  The values
are the same and so is the arithmetic, so every result must equal the per-node path's bit for bit
(tolerance 0): Fapply, residual and smoother sweeps in FP64 and FP32, and whole solves (iteration
counts and solutions), single level and two-level AMR with ghost nodes."""
import ctypes as C

import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, microstructure, models
from anisotropicfracture_gb300.elastic import Elastic, Field, Linear, level_desc
from helpers import bc_pull_z, bc_random
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _descs(Ls):
    return [level_desc(tuple(L.dom_hi[d] for d in range(3)), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx))
            for L in Ls]


def _lo(L):
    return tuple(L.lo[d] - L.ng for d in range(3))


def _poly(Ls, ngr=8, seed=3):
    seeds = microstructure.voronoi_seeds(ngr, seed)
    tab = models.cubic(1.68, 1.21, 0.75, models.random_rotations(ngr, np.random.default_rng(seed + 1)))
    gids, Cs = [], []
    for L in Ls:
        lo = [L.lo[d] - L.ng for d in range(3)]
        hi = [L.hi[d] + L.ng for d in range(3)]
        g = microstructure.voronoi_grain_ids(lo, hi, tuple(L.dx), seeds).astype(np.int32)
        gids.append(np.ascontiguousarray(g[None]))
        Cs.append(np.ascontiguousarray(np.moveaxis(tab[g], -1, 0)))
    return gids, Cs, tab


def _ops(Ls, bc, gids, Cs, tab):
    a = Elastic(_descs(Ls), models.MAJORMINOR)
    b = Elastic(_descs(Ls), models.MAJORMINOR)
    for l, L in enumerate(Ls):
        a.SetModel(l, Field(Cs[l], _lo(L)))
        b.SetModelGrains(l, Field(gids[l], _lo(L)), tab)
    for op in (a, b):
        op.SetBC(bc)
        op.SetUniform(False)
        op.prepareForSolve()
    return a, b


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_grain_kernels_equal_per_node_kernels(precision):
    Ls = [po.level((12, 10, 14))]
    rng = np.random.default_rng(5)
    gids, Cs, tab = _poly(Ls)
    bc = bc_random(rng)
    a, b = _ops(Ls, bc, gids, Cs, tab)
    dt = np.float64 if precision == "fp64" else np.float32

    def dev(x):
        return torch.from_numpy(np.ascontiguousarray(x)).cuda()

    u = dev(rng.standard_normal((3,) + Ls[0].shape).astype(dt))
    rhs = dev(rng.standard_normal((3,) + Ls[0].shape).astype(dt))
    fa, fb = torch.zeros_like(u), torch.zeros_like(u)
    a.Fapply(0, 0, Field(fa), Field(u))
    b.Fapply(0, 0, Field(fb), Field(u))
    torch.cuda.synchronize()
    assert torch.equal(fa, fb)
    if precision == "fp64":
        ra, rb = torch.zeros_like(u), torch.zeros_like(u)
        na = a.Residual(0, 0, Field(ra), Field(u), Field(rhs))
        nb = b.Residual(0, 0, Field(rb), Field(u), Field(rhs))
        torch.cuda.synchronize()
        assert torch.equal(ra, rb) and na == nb
        xa, xb = u.clone(), u.clone()
        a.Fsmooth(0, 0, Field(xa), Field(rhs))
        b.Fsmooth(0, 0, Field(xb), Field(rhs))
        torch.cuda.synchronize()
        assert torch.equal(xa, xb)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nlev", [1, 2])
def test_grain_solves_equal_per_node_solves(precision, nlev):
    Ls = po.amr_levels(16, nlev)
    gids, Cs, tab = _poly(Ls, ngr=10, seed=7)
    bc = bc_pull_z()
    bs = [po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape)) for L in Ls]
    a, b = _ops(Ls, bc, gids, Cs, tab)
    outs = []
    for op in (a, b):
        s = Linear(op)
        s.setMaxFmgIter(0)
        s.opts.bottom, s.opts.nu1, s.opts.nu2 = 0, 1, 1
        s.opts.inner_cycles = 2
        s.setPrecision(precision)
        xs = [np.zeros_like(x) for x in bs]
        s.solve([Field(x, _lo(L)) for x, L in zip(xs, Ls)], [Field(x, _lo(L)) for x, L in zip(bs, Ls)], 1e-8, 0.0)
        outs.append((xs, s.stats.iters, s.stats.converged))
    (xa, ia, ca), (xb, ib, cb) = outs
    assert ca and cb and ia == ib
    for p, q in zip(xa, xb):
        assert np.array_equal(p, q)
    a.close()
    b.close()


def test_bad_grain_ids_are_rejected():
    Ls = [po.level(8)]
    gids, Cs, tab = _poly(Ls, ngr=4)
    gids[0][0, 1, 2, 3] = 4
    op = Elastic(_descs(Ls), models.MAJORMINOR)
    with pytest.raises(_lib.AeError) as e:
        op.SetModelGrains(0, Field(gids[0]), tab)
    assert e.value.code == _lib.AE_ERR_ARG
    op.close()
