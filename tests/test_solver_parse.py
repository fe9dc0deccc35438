"""The solver mirrors' ParmParse keys (host only: no operator, no device): Linear::Parse
(src/Solver/Nonlocal/Linear.H:121-140) and Newton<T>::Parse (src/Solver/Nonlocal/Newton.H:342-347)."""
from anisotropicfracture_gb300.elastic import Linear, Newton


def test_linear_defaults_and_keys():
    s = Linear(None)
    assert s.opts.max_fmg_iter == 100000000 and s.opts.bottom == 1  # F-cycles, BiCGStab bottom
    Linear.Parse(s, {"max_iter": "50", "bottom_max_iter": "20", "max_fmg_iter": "0", "verbose": "2",
                     "bottom_solver": "cg", "pre_smooth": "3", "post_smooth": "4", "tol_rel": "1e-9"})
    o = s.opts
    assert (o.max_iter, o.bottom_max_iter, o.max_fmg_iter, o.verbose, o.bottom, o.nu1, o.nu2) == (50, 20, 0, 2, 0, 3, 4)
    assert s.m_tol_rel == 1e-9
    assert o.fixed_iter == 0
    Linear.Parse(s, {"fixed_iter": "6"})  # Linear.H:132-133
    assert s.opts.fixed_iter == 6


def test_newton_adds_nriters():
    s = Newton(None)
    assert s.m_nriters == 1
    Newton.Parse(s, {"nriters": "5", "max_iter": "7", "precision": "mixed"})
    assert s.m_nriters == 5 and s.opts.max_iter == 7 and s.opts.precision == 1
