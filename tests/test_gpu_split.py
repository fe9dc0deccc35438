"""The split FP32 sweep on grain-map levels (ae_split.cu: a TMA-staged tiled kernel over the
interior box plus the per-node code over the boundary shell) against the one-pass per-node sweep
(AE_SPLIT=0, read when an operator is created).  Every node is computed with the per-node sweep's
own arithmetic, so the results must be equal bit for bit (tolerance 0): FP32 Fsmooth on a single
level of 49 x 41 x 53 nodes (partial tiles, anisotropic spacing; the launch count shows the split
ran) and on refined patches with ghost layers
(inside the domain, and touching its low faces), m_uniform on and off, random BC tables, and
whole mixed-precision solves.  Also: the padded row pitch of the level arrays (AE_PAD=0: dense)
changes no result."""
import os

import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, microstructure, models
from anisotropicfracture_gb300.elastic import Elastic, Field, Linear, level_desc
from helpers import bc_random, polycrystal_amr
from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _single():
    """One level of 49 x 41 x 53 nodes with anisotropic spacing: partial tiles in every direction.
    Its cell counts are even, so it coarsens and keeps the padded row pitch the split sweep needs
    (the coarsest level of AMR level 0 stays dense and runs the per-node kernels)."""
    return po.level((48, 40, 52), dx=(1.0 / 48, 1.2 / 40, 0.9 / 52))


def _launches():
    return int(_lib.load().ae_kernel_launches())


def _descs(Ls):
    return [level_desc(tuple(L.dom_hi[d] for d in range(3)), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx))
            for L in Ls]


def _lo(L):
    return tuple(L.lo[d] - L.ng for d in range(3))


def _grains(Ls, ngr=12, seed=9):
    seeds = microstructure.voronoi_seeds(ngr, seed)
    tab = models.cubic(1.68, 1.21, 0.75, models.random_rotations(ngr, np.random.default_rng(seed + 1)))
    gids = []
    for L in Ls:
        lo = [L.lo[d] - L.ng for d in range(3)]
        hi = [L.hi[d] + L.ng for d in range(3)]
        g = microstructure.voronoi_grain_ids(lo, hi, tuple(L.dx), seeds).astype(np.int32)
        gids.append(np.ascontiguousarray(g[None]))
    return gids, tab


def _op(split, Ls, bc, gids, tab, uniform, pad=True):
    os.environ["AE_SPLIT"] = "1" if split else "0"
    os.environ["AE_PAD"] = "1" if pad else "0"
    try:
        op = Elastic(_descs(Ls), models.MAJORMINOR)
    finally:
        os.environ.pop("AE_SPLIT", None)
        os.environ.pop("AE_PAD", None)
    for l, L in enumerate(Ls):
        op.SetModelGrains(l, Field(gids[l], _lo(L)), tab)
    op.SetBC(bc)
    op.SetUniform(uniform)
    op.prepareForSolve()
    return op


def _fsmooth_counted(op, a, L, x, b, sweeps, fs=None):
    """_fsmooth (or fs), and the kernels it launched (after a call without sweeps, which makes
    the FP32 copies)."""
    fs = fs or _fsmooth
    fs(op, a, L, x, b, 0)
    n0 = _launches()
    out = fs(op, a, L, x, b, sweeps)
    return out, _launches() - n0


def _fsmooth(op, a, L, x, b, sweeps):
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    bd = torch.from_numpy(b.astype(np.float32)).cuda()
    op.Fsmooth(a, 0, Field(xd, _lo(L)), Field(bd, _lo(L)), sweeps, 2.0 / 3.0)
    torch.cuda.synchronize()
    return xd.cpu().numpy()


@pytest.mark.parametrize("uniform", [False, True])
def test_split_sweep_equals_per_node_single_level(uniform):
    Ls = [_single()]
    gids, tab = _grains(Ls)
    rng = np.random.default_rng(1)
    bc = bc_random(rng)
    x = rng.standard_normal((3,) + Ls[0].shape)
    b = rng.standard_normal((3,) + Ls[0].shape)
    ref, n_ref = _fsmooth_counted(_op(False, Ls, bc, gids, tab, uniform, pad=False), 0, Ls[0], x, b, 3)
    got, n_split = _fsmooth_counted(_op(True, Ls, bc, gids, tab, uniform), 0, Ls[0], x, b, 3)
    assert np.array_equal(got, ref), int((got != ref).sum())
    # the split ran: two launches per sweep (tiled kernel and list) instead of one
    assert n_split - n_ref == 3, (n_split, n_ref)


@pytest.mark.parametrize("where", ["inside", "low_corner"])
def test_split_sweep_equals_per_node_on_a_refined_patch(where):
    if where == "inside":
        Ls, _, bc, _ = polycrystal_amr(24, 2)
    else:  # a patch whose ghost layers reach past the domain's low faces
        Ls = [po.level(24), po.level(48, lo=(0, 0, 0), hi=(24, 24, 24), ng=2)]
        bc = bc_random(np.random.default_rng(4))
    gids, tab = _grains(Ls)
    rng = np.random.default_rng(2)
    for a, L in enumerate(Ls):
        x = rng.standard_normal((3,) + L.shape)
        b = rng.standard_normal((3,) + L.shape)
        ref = _fsmooth(_op(False, Ls, bc, gids, tab, False, pad=False), a, L, x, b, 2)
        got = _fsmooth(_op(True, Ls, bc, gids, tab, False), a, L, x, b, 2)
        assert np.array_equal(got, ref), (a, int((got != ref).sum()))


@pytest.mark.parametrize("nlev", [1, 2])
def test_split_sweep_mixed_solve_equals_per_node(nlev):
    Ls, Cs, bc, bs = polycrystal_amr(24, nlev)
    gids, tab = _grains(Ls)
    out = []
    for split, pad in ((False, False), (True, True)):
        op = _op(split, Ls, bc, gids, tab, False, pad)
        s = Linear(op)
        s.setMaxFmgIter(0)
        s.setBottomSolver("cg")
        s.setPreSmooth(1)
        s.setPostSmooth(1)
        s.setPrecision("mixed")
        s.opts.inner_cycles = 4
        xs = [np.zeros_like(b) for b in bs]
        s.solve([Field(x, _lo(L)) for x, L in zip(xs, Ls)], [Field(b, _lo(L)) for b, L in zip(bs, Ls)], 1e-8, 0.0)
        assert s.stats.converged
        out.append((s.stats.iters, xs))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)


def _fsmooth64(op, a, L, x, b, sweeps):
    xd = torch.from_numpy(x.astype(np.float64)).cuda()
    bd = torch.from_numpy(b.astype(np.float64)).cuda()
    op.Fsmooth(a, 0, Field(xd, _lo(L)), Field(bd, _lo(L)), sweeps, 2.0 / 3.0)
    torch.cuda.synchronize()
    return xd.cpu().numpy()


@pytest.mark.parametrize("uniform", [False, True])
def test_split_fp64_sweep_equals_per_node(uniform):
    """The FP64 split sweep (the reference's damped-Jacobi update, D read from its own tile)
    against the one-pass FP64 sweep, bit for bit: a single level and a refined patch."""
    rng = np.random.default_rng(7)
    Ls = [_single()]
    gids, tab = _grains(Ls)
    bc = bc_random(rng)
    x = rng.standard_normal((3,) + Ls[0].shape)
    b = rng.standard_normal((3,) + Ls[0].shape)
    ref, n_ref = _fsmooth_counted(_op(False, Ls, bc, gids, tab, uniform, pad=False), 0, Ls[0], x, b, 3, _fsmooth64)
    got, n_split = _fsmooth_counted(_op(True, Ls, bc, gids, tab, uniform), 0, Ls[0], x, b, 3, _fsmooth64)
    assert np.array_equal(got, ref), int((got != ref).sum())
    assert n_split - n_ref == 3, (n_split, n_ref)
    Ls, _, bc, _ = polycrystal_amr(24, 2)
    gids, tab = _grains(Ls)
    for a, L in enumerate(Ls):
        x = rng.standard_normal((3,) + L.shape)
        b = rng.standard_normal((3,) + L.shape)
        ref = _fsmooth64(_op(False, Ls, bc, gids, tab, uniform, pad=False), a, L, x, b, 2)
        got = _fsmooth64(_op(True, Ls, bc, gids, tab, uniform), a, L, x, b, 2)
        assert np.array_equal(got, ref), (a, int((got != ref).sum()))


@pytest.mark.parametrize("nlev", [1, 2])
def test_split_fp64_solve_equals_per_node(nlev):
    """Whole FP64 solves (every sweep and residual of the grain-map levels split) equal the
    one-pass solves bit for bit, with the same iteration count."""
    Ls, Cs, bc, bs = polycrystal_amr(24, nlev)
    gids, tab = _grains(Ls)
    out = []
    for split in (False, True):
        op = _op(split, Ls, bc, gids, tab, False, split)
        s = Linear(op)
        s.setMaxFmgIter(0)
        s.setBottomSolver("cg")
        s.setPrecision("fp64")
        xs = [np.zeros_like(b) for b in bs]
        s.solve([Field(x, _lo(L)) for x, L in zip(xs, Ls)], [Field(b, _lo(L)) for b, L in zip(bs, Ls)], 1e-8, 0.0)
        assert s.stats.converged
        out.append((s.stats.iters, xs))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_split_fapply_equals_per_node(dtype):
    """Fapply through the split kernels (staged through the level's buffers) equals the one-pass
    per-node Fapply over the caller's fabs, bit for bit, on a single level and a refined patch."""
    rng = np.random.default_rng(12)
    for Ls, bc in (([_single()], bc_random(rng)),
                   (polycrystal_amr(24, 2)[0], bc_random(rng))):
        gids, tab = _grains(Ls)
        for a, L in enumerate(Ls):
            x = rng.standard_normal((3,) + L.shape).astype(dtype)
            outs = []
            for split in (False, True):
                op = _op(split, Ls, bc, gids, tab, False, pad=split)
                xd = torch.from_numpy(x).cuda()
                fd = torch.zeros_like(xd)
                op.Fapply(a, 0, Field(fd, _lo(L)), Field(xd, _lo(L)))
                torch.cuda.synchronize()
                outs.append(fd.cpu().numpy())
                op.close()
            assert np.array_equal(outs[0], outs[1]), (a, int((outs[0] != outs[1]).sum()))


def test_padded_pitch_changes_no_fp64_result():
    """The FP64 solve on the padded layout equals the dense layout bit for bit."""
    Ls, Cs, bc, bs = polycrystal_amr(24, 2)
    gids, tab = _grains(Ls)
    sols = []
    for pad in (False, True):
        op = _op(False, Ls, bc, gids, tab, False, pad)
        s = Linear(op)
        s.setMaxFmgIter(0)
        s.setPrecision("fp64")
        xs = [np.zeros_like(b) for b in bs]
        s.solve([Field(x, _lo(L)) for x, L in zip(xs, Ls)], [Field(b, _lo(L)) for b, L in zip(bs, Ls)], 1e-8, 0.0)
        sols.append((s.stats.iters, xs))
    assert sols[0][0] == sols[1][0]
    for a, b in zip(sols[0][1], sols[1][1]):
        assert np.array_equal(a, b)

