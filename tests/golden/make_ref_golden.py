"""Writes tests/golden/ref_ops.npz: seeded inputs and the outputs of the REFERENCE'S OWN CODE for
the per-node operator functions.

The outputs come from oracle/_ref/libref.so, which oracle/refshim/build_ref.py compiles from the
reference tree: its Elastic<T>::Fapply / Diagonal / Strain / Stress / Energy /
averageDownCoeffsSameAmrLevel and Operator<Node>::Fsmooth / restriction / interpolation
definitions, cut verbatim from src/Operator/Elastic.cpp and src/Operator/Operator.cpp, with its
unmodified model, tensor, stencil and BC headers (BC::Operator::Elastic<T>::Init included), built
against stand-ins for AMReX and Eigen (oracle/refshim/include).  It therefore needs the reference
tree (/root/reference/src, or $AE_REFERENCE_SRC) and runs only where that is present; the
fixtures it writes are committed so that the checks run anywhere.

Cases (inputs are multiples of 1/64, or of 1/1024 for the cubic tables: exact and compressible):
  box_<model>    an 8 x 6 x 10-cell level, spacing (0.1, 0.15, 0.08), random BC table mixing
                 displacement / traction / Neumann rows with random values:
                 fapply, fapply_uniform, diag, fsmooth (one Fsmooth call, 2 sweeps, from the
                 reference's own diagonal), stress, stress_voigt, energy, coarse_C
                 (averageDownCoeffsSameAmrLevel onto the 4 x 3 x 5-cell level)
  patch_<model>  a refined patch: nodes (2..6, 2..4, 2..6) of an 8-cell domain, 2 ghost layers,
                 touching no domain face: fapply, diag, fsmooth
  edge_<model>   a patch with ghosts that touches the domain's low x and high z faces: fapply,
                 diag, fsmooth
  fields         strain, strain_voigt (model-free), restrict, interp, bc_init, bc_init_homog on
                 the box level
  cubic          Linear::Cubic::Define(1.68, 1.21, 0.75, R) for 6 rotations: cubic_R, cubic_tabs
  <lname>_major  the 45-slot Sym::Major kind (Elastic<Model::Solid::Elastic::NeoHookean>), its
                 per-node tangent DDW(F) from the reference's NeoHookean at F = I + (multiples of
                 1/64 in [-1/8, 1/8)), mu = 1.25, kappa = 2.5, rounded to multiples of 1/1024
                 (a tangent field with the major symmetry only): the cases above without
                 Stress / Energy (which read a linear model)
  neo            NeoHookean::W / DW / DDW (mu = 1.3, kappa = 2.7) at 48 deformation gradients:
                 neo_F, neo_w, neo_dw, neo_ddw (45 slots)

Regenerate with:  python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from anisotropicfracture_gb300 import models  # noqa: E402
from helpers import golden_stiffness  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(HERE, "ref_ops.npz")
CELLS = (8, 6, 10)
DX = (0.1, 0.15, 0.08)
D, T, N = 0, 1, 3
NAMES = [(models.ISOTROPIC, "iso"), (models.MAJORMINOR, "mm"), (models.DIAGONAL, "diag"), (models.MAJOR, "major")]


def q(rng, shape, lo=-64, hi=64):
    """Random multiples of 1/64 in [lo/64, hi/64)."""
    return rng.integers(lo, hi, size=shape).astype(np.float64) / 64.0


def coeffs(model, shape, rng):
    """Per-node stiffness and the parts it is stored as (see helpers.golden_stiffness)."""
    if model == models.ISOTROPIC:
        C = np.ascontiguousarray(np.stack([1.0 + q(rng, shape, 0, 64), 0.5 + q(rng, shape, 0, 64)]))
        return C, {"C": C}
    if model == models.DIAGONAL:
        C = np.ascontiguousarray(0.5 + q(rng, (9,) + shape, 0, 64))
        return C, {"C": C}
    if model == models.MAJOR:
        from oracle.refshim import pyref
        F = np.eye(3) + q(rng, shape + (3, 3), -8, 8)
        ddw = pyref.neohookean(1.25, 2.5, F)[2].reshape(shape + (45,))
        C = np.ascontiguousarray(np.moveaxis(np.round(ddw * 1024.0) / 1024.0, -1, 0))
        return C, {"C": C}
    Rs = models.random_rotations(4, rng)
    tabs = np.round(models.cubic(1.68, 1.21, 0.75, Rs) * 1024.0) / 1024.0
    gid = rng.integers(0, 4, size=shape).astype(np.uint8)
    scale = 1.0 + q(rng, shape, -8, 8)
    parts = {"tabs": tabs, "gid": gid, "scale": scale}
    return golden_stiffness(parts), parts


def bc_table(rng):
    return rng.choice([D, T, N], size=(26, 3)).astype(np.int32), q(rng, (26, 3))


def levels():
    """name -> oracle level description"""
    return {"box": po.level(CELLS, dx=DX),
            "patch": po.level(8, lo=(2, 2, 2), hi=(6, 4, 6), ng=2),
            "edge": po.level(8, lo=(0, 2, 4), hi=(4, 6, 8), ng=2)}


def make():
    from oracle.refshim import pyref
    out = {"cells": np.array(CELLS, np.int32), "dx": np.array(DX)}
    Ls = levels()
    for lname, L in Ls.items():
        out[lname + "_level"] = np.array(list(L.dom_lo) + list(L.dom_hi) + list(L.lo) + list(L.hi) + [L.ng],
                                         np.int32)
        out[lname + "_dxs"] = np.array(list(L.dx))
    for model, name in NAMES:
        for lname, L in Ls.items():
            rng = np.random.default_rng(3000 + 10 * model + len(lname))
            C, parts = coeffs(model, L.shape, rng)
            bt, bv = bc_table(rng)
            u, x, b = (q(rng, (3,) + L.shape) for _ in range(3))
            dg = pyref.diagonal(L, model, C, bt, bv)
            p = "%s_%s_" % (lname, name)
            out.update({p + k: v for k, v in parts.items()})
            out.update({p + "model": np.int32(model), p + "bc_type": bt, p + "bc_val": bv, p + "u": u, p + "x": x,
                        p + "b": b, p + "fapply": pyref.fapply(L, model, C, bt, u, bcval=bv), p + "diag": dg,
                        p + "fsmooth": pyref.fsmooth(L, model, C, bt, dg, x, b, bcval=bv)})
            if lname == "box":
                Lc = po.coarsen(L)
                out.update({p + "fapply_uniform": pyref.fapply(L, model, C, bt, u, True, bcval=bv),
                            p + "coarse_C": pyref.average_down_coeffs(L, Lc, model, C)})
                if model != models.MAJOR:
                    out.update({p + "stress": pyref.fields(L, model, C, "stress", u),
                                p + "stress_voigt": pyref.fields(L, model, C, "stress", u, True),
                                p + "energy": pyref.fields(L, model, C, "energy", u)})
    rng = np.random.default_rng(3100)
    L = Ls["box"]
    Lc = po.coarsen(L)
    u, x = q(rng, (3,) + L.shape), q(rng, (3,) + L.shape)
    crse = q(rng, (3,) + Lc.shape)
    bt, bv = bc_table(rng)
    r0 = q(rng, (3,) + L.shape)
    out.update({"fields_u": u, "fields_x": x, "fields_crse": crse, "fields_bc_type": bt, "fields_bc_val": bv,
                "fields_r0": r0,
                "fields_strain": pyref.fields(L, models.ISOTROPIC, np.ones((2,) + L.shape), "strain", u),
                "fields_strain_voigt": pyref.fields(L, models.ISOTROPIC, np.ones((2,) + L.shape), "strain", u, True),
                "fields_restrict": pyref.restrict(Lc, L, u),
                "fields_interp": pyref.interp_add(L, Lc, x, crse),
                "fields_bc_init": pyref.bc_init(L, bt, bv, r0),
                "fields_bc_init_homog": pyref.bc_init(L, bt, bv, r0, True)})
    Rs = models.random_rotations(6, np.random.default_rng(3200))
    out["cubic_R"] = Rs
    out["cubic_tabs"] = np.stack([pyref.cubic_define(1.68, 1.21, 0.75, R) for R in Rs])
    F = np.eye(3) + 0.25 * np.random.default_rng(3300).standard_normal((48, 3, 3))
    w, dw, ddw = pyref.neohookean(1.3, 2.7, F)
    out.update({"neo_F": F, "neo_w": w, "neo_dw": dw, "neo_ddw": ddw})
    return out


if __name__ == "__main__":
    from oracle.refshim import build_ref
    if not build_ref.available():
        sys.exit("the reference tree is needed: %s" % build_ref.reference_src())
    np.savez_compressed(OUT, **make())
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
