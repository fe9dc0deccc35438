"""The outermost ghost ring of a refined patch in the FP64 composite solve (oracle, CPU).

The ring of grow(valid, 2) has no equation: the composite iteration only adds coarse corrections
interpolated to it (src/Operator/Operator.cpp:556-624).  Started from zero, the ring therefore
holds the interpolation of the coarse solution.  The mixed-precision solve relies on this: it
rebuilds the ring's increments from the coarse correction in FP64 instead of keeping the FP32
cycle's rounded interpolation."""
import numpy as np
import pytest

from oracle import pyoracle as po
from helpers import polycrystal_amr


def _interp(c, lo0, n, i, j, k):
    """Coarse field c (storage origin lo0) interpolated to fine node (i, j, k): the mean of the
    coarse nodes around it (1, 2, 4 or 8 of them by the parity of i, j, k)."""
    I, J, K = i // 2, j // 2, k // 2
    vals = [c[n, K + dk - lo0[2], J + dj - lo0[1], I + di - lo0[0]]
            for di in range(1 + (i & 1)) for dj in range(1 + (j & 1)) for dk in range(1 + (k & 1))]
    return sum(vals) / len(vals)


@pytest.mark.parametrize("n", [12, 16])
def test_fp64_ring_is_the_interpolated_coarse_solution(n):
    Ls, Cs, bc, bs = polycrystal_amr(n, 2)
    x, st, rc = po.solve_amr(Ls, po.ORC_MAJORMINOR, Cs, bc.type, [np.zeros_like(b) for b in bs], bs, 1e-10, 0.0)
    assert rc == 0
    L0, L1 = Ls
    lo0 = [L0.lo[d] - L0.ng for d in range(3)]
    lo1 = [L1.lo[d] - L1.ng for d in range(3)]
    sh = x[1].shape[1:]
    worst, checked = 0.0, 0
    for kk in range(sh[0]):
        for jj in range(sh[1]):
            for ii in range(sh[2]):
                if not (kk in (0, sh[0] - 1) or jj in (0, sh[1] - 1) or ii in (0, sh[2] - 1)):
                    continue
                i, j, k = ii + lo1[0], jj + lo1[1], kk + lo1[2]
                for comp in range(3):
                    worst = max(worst, abs(x[1][comp, kk, jj, ii] - _interp(x[0], lo0, comp, i, j, k)))
                    checked += 1
    assert checked > 0
    assert worst <= 1e-14 * np.abs(x[1]).max()
