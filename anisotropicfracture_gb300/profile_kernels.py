"""Kernel timing tool: one level of the seeded cubic polycrystal, one kernel launched
back to back on the solver's own buffers, duration from CUDA events (ae_profile_kernel).

    python -m anisotropicfracture_gb300.profile_kernels --cells 128 --kernel jacobi --precision fp32

Kernels: fapply, jacobi, residual, restrict, interp.  Prints one JSON line with the average
launch time and the algorithmic bandwidth (canonical bytes per node / time).  Also the
workload for ncu captures of a single kernel (-k regex:<mangled name> -s 1 -c N).

--tangent: instead of the polycrystal, the 45-slot Sym::Major stiffness of a NeoHookean tangent
DDW(I + grad u) at a small random displacement, set by ae_newton_neohookean.
"""
import argparse
import ctypes as C
import json
import os
import sys

import numpy as np

KERNELS = {"fapply": 0, "jacobi": 1, "residual": 2, "restrict": 3, "interp": 4}
# canonical algorithmic bytes per (fine) node, cubic stiffness: {precision: bytes}
BYTES = {"fapply": {8: 216, 4: 108}, "jacobi": {8: 264, 4: 132}, "residual": {8: 240, 4: 120},
         "restrict": {8: 27, 4: 13.5}, "interp": {8: 51, 4: 25.5}}
# the same kernels on a grain map: the stiffness is a 2-byte id per node
GRAIN_BYTES = {"fapply": {8: 50, 4: 26}, "jacobi": {8: 122, 4: 50}, "residual": {8: 74, 4: 38}}
# the same kernels on a 45-slot Sym::Major stiffness
MAJOR_BYTES = {"fapply": {8: 408, 4: 204}, "jacobi": {8: 456, 4: 228}, "residual": {8: 432, 4: 216},
               "restrict": {8: 27, 4: 13.5}, "interp": {8: 51, 4: 25.5}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=128)
    ap.add_argument("--kernel", default="jacobi", choices=sorted(KERNELS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--mglev", type=int, default=0)
    ap.add_argument("--grains", type=int, default=64)
    ap.add_argument("--grain-map", action="store_true",
                    help="give the stiffness as grain ids + table (ae_op_set_model_grains)")
    ap.add_argument("--tangent", action="store_true",
                    help="a NeoHookean tangent stiffness (45 Sym::Major slots per node)")
    args = ap.parse_args(argv)

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    from anisotropicfracture_gb300 import _lib, microstructure, models
    from anisotropicfracture_gb300.elastic import BCElastic, Elastic, Field, level_desc

    n = args.cells
    bc = BCElastic()
    for f in ["XLO", "XHI", "YLO", "YHI", "XLO_YLO", "XLO_YHI", "XHI_YLO", "XHI_YHI"]:
        for d in range(3):
            bc.Set(f, d, bc.Traction, 0.0)
    if args.tangent:
        op = Elastic([level_desc(n)], models.MAJOR)
        op.SetBC(bc)
        rng = np.random.default_rng(3)
        u = 0.01 / n * rng.standard_normal((3,) + (n + 1,) * 3)
        rhs = np.zeros_like(u)
        op.NewtonNeoHookean(0, Field(rhs), Field(u), Field(np.zeros_like(u)), models.NeoHookean(1.0, 2.5))
    else:
        Cf, gid, table = microstructure.cubic_polycrystal((0, 0, 0), (n, n, n), (1.0 / n,) * 3, nseeds=args.grains)
        op = Elastic([level_desc(n)], models.MAJORMINOR)
        if args.grain_map:
            op.SetModelGrains(0, Field(np.ascontiguousarray(gid[None].astype(np.int32))), table)
        else:
            op.SetModel(0, Field(Cf))
    op.SetBC(bc)
    op.SetUniform(False)
    op.prepareForSolve()
    lib = _lib.load()
    prec = 1 if args.precision == "fp32" else 0
    ms = C.c_double(0.0)
    _lib.check(lib.ae_profile_kernel(op.handle, KERNELS[args.kernel], 0, args.mglev, prec, args.reps, C.byref(ms)))
    nodes = (n // 2 ** args.mglev + 1) ** 3
    table = GRAIN_BYTES if (args.grain_map and args.mglev == 0 and args.kernel in GRAIN_BYTES) else BYTES
    if args.tangent:
        table = MAJOR_BYTES
    nbytes = table[args.kernel][4 if prec else 8] * nodes
    print(json.dumps({"kernel": args.kernel, "precision": args.precision, "cells": n, "mglev": args.mglev,
                      "grain_map": bool(args.grain_map), "tangent": bool(args.tangent), "nodes": nodes, "ms_per_launch": ms.value,
                      "bytes_per_node": table[args.kernel][4 if prec else 8],
                      "algorithmic_GBps": nbytes / (ms.value * 1e-3) / 1e9}))
    op.close()


if __name__ == "__main__":
    main()
