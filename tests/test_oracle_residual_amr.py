"""The oracle's stand-alone composite residual (orc_residual_amr) equals the composite residual its
MLMG restatement computes inside a solve, for one, two and three AMR levels.  The benchmark uses
it to have the oracle evaluate b - A x for the GPU's final solutions."""
import numpy as np
import pytest

from helpers import polycrystal_amr
from oracle import pyoracle as po


@pytest.mark.parametrize("nlev", [1, 2, 3])
def test_residual_amr_equals_solver_initial_residual(nlev):
    Ls, Cs, bc, bs = polycrystal_amr(16, nlev)
    rng = np.random.default_rng(nlev)
    us = [1e-3 * rng.standard_normal(b.shape) for b in bs]
    _, st, _ = po.solve_amr(Ls, po.ORC_MAJORMINOR, Cs, bc.type, us, bs, 1e-30, 0.0, max_iter=0)
    rn = po.residual_amr(Ls, po.ORC_MAJORMINOR, Cs, bc.type, us, bs)
    assert rn == st.res0
    if nlev == 1:
        _, ref = po.residual(Ls[0], po.ORC_MAJORMINOR, Cs[0], bc.type, us[0], bs[0])
        assert rn == ref
