"""The oracle's composite solve with several patches per AMR level (an AMReX BoxArray of separated
boxes): the reference's multi-level known-answer tests (src/Test/Operator/Elastic_UniaxialTest.cpp,
Elastic_TrigTest.cpp) on hierarchies whose refined levels are two or more patches, the solution
independent of the order the patches are listed in, and malformed hierarchies refused."""
import numpy as np
import pytest

from oracle import pyoracle as po
from test_oracle_known_answers import bc_uniaxial_x


def patches(n=32, three=False):
    """Level 0: n^3 cells.  Level 1: two separated patches of the 2n domain.  With three, level 2
    refines one patch inside each level-1 patch."""
    Ls = [po.level(n),
          po.level(2 * n, lo=(8, 8, 8), hi=(24, 24, 24), ng=2),
          po.level(2 * n, lo=(36, 8, 28), hi=(56, 24, 52), ng=2)]
    if three:
        Ls += [po.level(4 * n, lo=(24, 24, 24), hi=(40, 40, 40), ng=2),
               po.level(4 * n, lo=(80, 24, 64), hi=(104, 40, 96), ng=2)]
    return Ls


def _valid(a, L):
    g = L.ng
    return a[(slice(None),) + (slice(g, a.shape[1] - g),) * 3] if g else a


def _uniaxial(Ls):
    bc = bc_uniaxial_x()
    bs, us, Cs, ex = [], [], [], []
    for L in Ls:
        X, Y, Z = po.node_coords(L)
        c = np.empty((2,) + L.shape)
        c[0], c[1] = 6.0, 2.6
        bs.append(po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape)))
        us.append(np.zeros((3,) + L.shape))
        Cs.append(c)
        ex.append(0.1 * X)
    return bc, bs, us, Cs, ex


@pytest.mark.parametrize("three", [False, True])
def test_uniaxial_on_patches(three):
    Ls = patches(three=three)
    bc, bs, us, Cs, ex = _uniaxial(Ls)
    u, st, rc = po.solve_amr(Ls, po.ORC_ISOTROPIC, Cs, bc.type, us, bs, 1e-10, 0.0)
    assert rc == 0 and st.converged
    err = max(np.abs(_valid(u[a], L)[0] - _valid(ex[a][None], L)[0]).max() for a, L in enumerate(Ls))
    assert err < 1e-8


def test_trig_on_patches():
    Ls = patches()
    bct, bcv = np.zeros((26, 3), np.int32), np.zeros((26, 3))
    bs, us, Cs, ex = [], [], [], []
    for L in Ls:
        X, Y, Z = po.node_coords(L)
        S3 = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
        b = np.zeros((3,) + L.shape)
        b[0] = S3
        bs.append(po.bc_init(L, bct, bcv, b))
        us.append(np.zeros_like(b))
        Cs.append(np.ones((9,) + L.shape))
        ex.append(-S3 / (3 * np.pi ** 2))
    u, st, rc = po.solve_amr(Ls, po.ORC_DIAGONAL, Cs, bct, us, bs, 1e-8, 1e-8, max_fmg_iter=0, bottom=0)
    assert rc == 0
    err = max(np.abs(_valid(u[a], L)[0] - _valid(ex[a][None], L)[0]).max() for a, L in enumerate(Ls))
    assert err / np.abs(ex[0]).max() < 0.02


def test_patch_order_does_not_matter():
    """Patches of a level are independent: listing them in another order gives the same solution
    bit for bit, with the same iteration count."""
    rng = np.random.default_rng(3)
    Ls = patches(three=True)
    bc = bc_uniaxial_x()
    Cs = [np.stack([1.0 + rng.random(L.shape), 0.5 + rng.random(L.shape)]) for L in Ls]
    bs = [po.bc_init(L, bc.type, bc.val, 0.1 * rng.standard_normal((3,) + L.shape)) for L in Ls]
    us = [np.zeros_like(b) for b in bs]
    u1, st1, rc1 = po.solve_amr(Ls, po.ORC_ISOTROPIC, Cs, bc.type, us, bs, 1e-9, 0.0, max_fmg_iter=0, bottom=0)
    perm = [0, 2, 1, 4, 3]
    u2, st2, rc2 = po.solve_amr([Ls[p] for p in perm], po.ORC_ISOTROPIC, [Cs[p] for p in perm], bc.type,
                                [us[p] for p in perm], [bs[p] for p in perm], 1e-9, 0.0, max_fmg_iter=0, bottom=0)
    assert rc1 == 0 and rc2 == 0 and st1.iters == st2.iters
    for k, p in enumerate(perm):
        assert np.array_equal(u2[k], u1[p])
    # the composite residual is the same function of the patches
    r1 = po.residual_amr(Ls, po.ORC_ISOTROPIC, Cs, bc.type, u1, bs)
    r2 = po.residual_amr([Ls[p] for p in perm], po.ORC_ISOTROPIC, [Cs[p] for p in perm], bc.type, u2,
                         [bs[p] for p in perm])
    assert r1 == r2


@pytest.mark.parametrize("bad", ["touching", "outside_parent", "same_domain_as_base"])
def test_malformed_hierarchies_are_refused(bad):
    n = 16
    if bad == "touching":  # storage boxes grow(valid, 2) overlap
        Ls = [po.level(n), po.level(2 * n, lo=(4, 4, 4), hi=(12, 12, 12), ng=2),
              po.level(2 * n, lo=(14, 4, 4), hi=(22, 12, 12), ng=2)]
    elif bad == "outside_parent":  # a level-2 patch that no level-1 patch contains
        Ls = [po.level(n), po.level(2 * n, lo=(4, 4, 4), hi=(12, 12, 12), ng=2),
              po.level(4 * n, lo=(40, 40, 40), hi=(48, 48, 48), ng=2)]
    else:
        Ls = [po.level(n), po.level(n, lo=(4, 4, 4), hi=(8, 8, 8), ng=2)]
    Cs = [np.ones((9,) + L.shape) for L in Ls]
    bs = [np.zeros((3,) + L.shape) for L in Ls]
    _, _, rc = po.solve_amr(Ls, po.ORC_DIAGONAL, Cs, np.zeros((26, 3), np.int32), [b.copy() for b in bs], bs)
    assert rc == -1
    with pytest.raises(RuntimeError):
        po.residual_amr(Ls, po.ORC_DIAGONAL, Cs, np.zeros((26, 3), np.int32), bs, bs)
