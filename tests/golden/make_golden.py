"""Writes tests/golden/elastic_ops.npz: seeded inputs and the oracle's outputs for the operator
functions on a small non-cubic box with anisotropic spacing, and one V-cycle solve.

The reference ships no golden vectors (its regression plotfiles live outside its repository) and
cannot be built without AMReX, Eigen and MPI, so these fixtures are the FP64 oracle's outputs,
committed so that a change of the oracle, of the platform it is built on, or of the GPU path shows
against a fixed record.  The oracle itself is pinned by the reference's own known-answer tests
(tests/test_oracle_known_answers.py).

Inputs are multiples of 1/64 (exact in FP32 and FP64, small when compressed).  Each case stores:
  model, cells, bc_type (26 x 3), bc_val (26 x 3), the per-node stiffness, u, x, b, crse
  fapply   = Elastic<T>::Fapply(u)                       src/Operator/Elastic.cpp:153-264
  diag     = Elastic<T>::Diagonal                        src/Operator/Elastic.cpp:266-352
  fsmooth  = Operator<Node>::Fsmooth(x, b), 2 sweeps     src/Operator/Operator.cpp:90-162
  resid    = b - Fapply(x), and its max-norm          src/Operator/Operator.cpp:842-852
  restrict = Operator<Node>::restriction(u)             src/Operator/Operator.cpp:454-554
  interp   = x + Operator<Node>::interpolation(crse)     src/Operator/Operator.cpp:556-624
  solve_u, solve_iters: V-cycle solve of the pull-along-z problem from zero to 1e-8

Regenerate with:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from anisotropicfracture_gb300 import models  # noqa: E402
from helpers import bc_pull_z, golden_stiffness  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(HERE, "elastic_ops.npz")
CELLS = (8, 6, 10)
SOLVE_CELLS = (8, 8, 8)
D, T, N = 0, 1, 3


def q(rng, shape, lo=-64, hi=64):
    """Random multiples of 1/64 in [lo/64, hi/64)."""
    return rng.integers(lo, hi, size=shape).astype(np.float64) / 64.0


def coeffs(model, shape, rng):
    """Per-node stiffness, returned with the parts it is stored as: the field itself for the
    isotropic and diagonal kinds; for the cubic kind a 4-grain slot table, a grain id per node and
    a per-node scale, C = table[gid] * scale (rebuilt by helpers.golden_stiffness)."""
    if model == models.ISOTROPIC:
        C = np.ascontiguousarray(np.stack([1.0 + q(rng, shape, 0, 64), 0.5 + q(rng, shape, 0, 64)]))
        return C, {"C": C}
    if model == models.DIAGONAL:
        C = np.ascontiguousarray(0.5 + q(rng, (9,) + shape, 0, 64))
        return C, {"C": C}
    # slot values rounded to multiples of 1/1024, so every product below is exact
    Rs = models.random_rotations(4, rng)
    tabs = np.round(models.cubic(1.68, 1.21, 0.75, Rs) * 1024.0) / 1024.0
    gid = rng.integers(0, 4, size=shape).astype(np.uint8)
    scale = 1.0 + q(rng, shape, -8, 8)
    parts = {"tabs": tabs, "gid": gid, "scale": scale}
    return golden_stiffness(parts), parts


def bc_table(rng):
    return rng.choice([D, T, N], size=(26, 3)).astype(np.int32), q(rng, (26, 3))


def make():
    out = {}
    for model, name in [(models.ISOTROPIC, "iso"), (models.MAJORMINOR, "mm"), (models.DIAGONAL, "diag")]:
        rng = np.random.default_rng(1000 + model)
        L = po.level(CELLS)
        C, parts = coeffs(model, L.shape, rng)
        bt, bv = bc_table(rng)
        u, x, b = (q(rng, (3,) + L.shape) for _ in range(3))
        dg = po.diagonal(L, model, C, bt)
        r, rn = po.residual(L, model, C, bt, x, b)
        Lc = po.coarsen(L)
        crse = q(rng, (3,) + Lc.shape)
        p = name + "_"
        out.update({p + k: v for k, v in parts.items()})
        out.update({p + "model": np.int32(model), p + "bc_type": bt, p + "bc_val": bv,
                    p + "u": u, p + "x": x, p + "b": b, p + "crse": crse,
                    p + "fapply": po.fapply(L, model, C, bt, u),
                    p + "fapply_uniform": po.fapply(L, model, C, bt, u, True),
                    p + "diag": dg,
                    p + "fsmooth": po.fsmooth(L, model, C, bt, dg, x, b, 2, 2.0 / 3.0),
                    p + "resid": r, p + "resid_norm": np.float64(rn),
                    p + "restrict": po.restrict(Lc, L, u),
                    p + "interp": po.interp_add(L, Lc, x, crse)})
    # a V-cycle solve of the pull-along-z problem (u = 0 on z = 0, u_z = 0.01 on z = 1) on 4 grains
    rng = np.random.default_rng(2000)
    L = po.level(SOLVE_CELLS)
    C, parts = coeffs(models.MAJORMINOR, L.shape, rng)
    bc = bc_pull_z()
    b = po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape))
    u, st, rc = po.solve(L, models.MAJORMINOR, C, bc.type, np.zeros_like(b), b, 1e-8, 0.0)
    assert rc == 0
    out.update({"solve_" + k: v for k, v in parts.items()})
    out.update({"solve_bc_type": bc.type.astype(np.int32), "solve_bc_val": bc.val,
                "solve_b": b, "solve_u": u, "solve_iters": np.int32(st.iters)})
    out["cells"] = np.array(CELLS, np.int32)
    out["solve_cells"] = np.array(SOLVE_CELLS, np.int32)
    return out


if __name__ == "__main__":
    np.savez_compressed(OUT, **make())
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
