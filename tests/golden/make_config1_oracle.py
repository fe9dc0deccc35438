"""Writes tests/golden/config1_oracle.npz: the FP64 oracle's full solve of the two-level polycrystal
workload (256^3 cells plus a ratio-2 patch over the central 1/8: two levels of 257^3 nodes, cubic
1.68 / 1.21 / 0.75 on 64 Voronoi grains, u = 0 on z = 0, u_z = 0.01 on z = 1, traction-free
lateral faces; V-cycle with one pre and one post smoother call of two damped-Jacobi sweeps, CG
bottom, 1e-8 relative residual), run on the host cores.

The solve takes tens of minutes on a CPU, too long for a benchmark run, so it is run once and a
subsample is committed:
  iters, res0, resfinal, target, hist   the oracle's iteration count and residual history
  stride                                 16: every 16th node in each direction
  sub0, sub1                             the solution at nodes (16 a, 16 b, 16 c) of each level's
                                         valid box, (3, 17, 17, 17) each
  seconds, threads                       wall time of the solve and the host threads it used
bench.py measures the displacement error of its GPU solutions at these nodes.

Run with:  python tests/golden/make_config1_oracle.py [threads]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "config1_oracle.npz")
STRIDE = 16


def main(threads=None):
    import bench
    from oracle import pyoracle as po
    if threads:
        po.set_threads(int(threads))
    levels, bc = bench.workload(256)
    Ls = [bench.oracle_level(L) for L in levels]
    Cs = [L["C"] for L in levels]
    bs = [bench.oracle_rhs(L, bc) for L in levels]
    us = [np.zeros_like(b) for b in bs]
    t0 = time.perf_counter()
    xs, st, rc = po.solve_amr(Ls, po.ORC_MAJORMINOR, Cs, bc.type, us, bs, 1e-8, 0.0, max_fmg_iter=0, bottom=0,
                          nu1=1, nu2=1, max_iter=400)
    secs = time.perf_counter() - t0
    assert rc == 0 and st.converged, "oracle solve did not converge"
    out = {"iters": np.int32(st.iters), "res0": np.float64(st.res0), "resfinal": np.float64(st.resfinal),
           "target": np.float64(st.target), "hist": np.array(st.hist[:st.iters]), "stride": np.int32(STRIDE),
           "seconds": np.float64(secs), "threads": np.int32(po.lib().orc_num_threads())}
    for a, (L, x) in enumerate(zip(levels, xs)):
        g = L["ng"]
        v = x[:, g:x.shape[1] - g, g:x.shape[2] - g, g:x.shape[3] - g] if g else x
        out["sub%d" % a] = np.ascontiguousarray(v[:, ::STRIDE, ::STRIDE, ::STRIDE])
    np.savez_compressed(OUT, **out)
    print(json.dumps({"iters": int(st.iters), "seconds": secs, "resfinal": st.resfinal, "target": st.target}))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
