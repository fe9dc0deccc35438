"""The oracle against the REFERENCE'S OWN CODE: tests/golden/ref_ops.npz holds outputs of the
reference's Elastic<T>::Fapply / Diagonal / Strain / Stress / Energy / averageDownCoeffsSameAmrLevel,
Operator<Node>::Fsmooth / restriction / interpolation, BC::Operator::Elastic<T>::Init and
Linear::Cubic::Define, compiled from the reference tree (tests/golden/make_ref_golden.py,
oracle/refshim/build_ref.py).  The oracle must reproduce every one of them bit for bit: it is
built with every multiply and add rounded separately, as the reference's build is, and follows
the reference's operation order.

Where the reference tree is present (not on a GPU machine), the fixtures are also regenerated from it
and must equal the committed ones, which shows where they came from."""
import os

import numpy as np
import pytest

from anisotropicfracture_gb300 import models
from helpers import golden_level, golden_prefixed
from oracle import pyoracle as po

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ops.npz")
NAMES = {"iso": models.ISOTROPIC, "mm": models.MAJORMINOR, "diag": models.DIAGONAL, "major": models.MAJOR}


@pytest.fixture(scope="module")
def z():
    return np.load(PATH)


def bitwise(a, b, what):
    assert a.shape == b.shape, what
    assert np.array_equal(a, b), "%s: %d nodes differ, max %.3e" % (what, int((a != b).sum()),
                                                                     float(np.abs(a - b).max()))


@pytest.mark.parametrize("lname", ["box", "patch", "edge"])
@pytest.mark.parametrize("name", list(NAMES))
def test_oracle_operator_is_bitwise_the_reference(z, lname, name):
    L = golden_level(z, lname)
    c = golden_prefixed(z, "%s_%s_" % (lname, name))
    model = NAMES[name]
    bt = c["bc_type"]
    bitwise(po.fapply(L, model, c["C"], bt, c["u"]), c["fapply"], "Fapply")
    D = po.diagonal(L, model, c["C"], bt)
    bitwise(D, c["diag"], "Diagonal")
    bitwise(po.fsmooth(L, model, c["C"], bt, D, c["x"], c["b"], 2, 2.0 / 3.0), c["fsmooth"], "Fsmooth")
    if lname == "box":
        bitwise(po.fapply(L, model, c["C"], bt, c["u"], True), c["fapply_uniform"], "Fapply m_uniform")
        bitwise(po.restrict(po.coarsen(L), L, c["C"]), c["coarse_C"], "averageDownCoeffsSameAmrLevel")
        if model != models.MAJOR:
            bitwise(po.stress(L, model, c["C"], c["u"]), c["stress"], "Stress")
            bitwise(po.stress(L, model, c["C"], c["u"], True), c["stress_voigt"], "Stress voigt")
            bitwise(po.energy(L, model, c["C"], c["u"]), c["energy"], "Energy")


def test_oracle_fields_and_transfers_are_bitwise_the_reference(z):
    L = golden_level(z, "box")
    Lc = po.coarsen(L)
    c = golden_prefixed(z, "fields_")
    bitwise(po.strain(L, c["u"]), c["strain"], "Strain")
    bitwise(po.strain(L, c["u"], True), c["strain_voigt"], "Strain voigt")
    bitwise(po.restrict(Lc, L, c["u"]), c["restrict"], "restriction")
    bitwise(po.interp_add(L, Lc, c["x"], c["crse"]), c["interp"], "interpolation")
    bitwise(po.bc_init(L, c["bc_type"], c["bc_val"], c["r0"]), c["bc_init"], "BC Init")
    bitwise(po.bc_init(L, c["bc_type"], c["bc_val"], c["r0"], True), c["bc_init_homog"], "BC Init homogeneous")


def test_neohookean_matches_the_reference(z):
    """The oracle's NeoHookean W / DW / DDW against the reference's NeoHookean.H evaluated at the
    same deformation gradients.  Not bitwise: the oracle takes det F and F^-1 from numpy's LU,
    the reference from Eigen's cofactor formulas; 1e-14 of each quantity's max-norm.  DDW is
    compared in the Sym::Major slots the reference stores, each holding the entry evaluated last
    in its (i, j, k, l) loop (the lower-triangle evaluation of A(3i+j, 3k+l))."""
    F = z["neo_F"]
    w, dw = po.neohookean_w(F, 1.3, 2.7), po.neohookean_dw(F, 1.3, 2.7)
    ddw = np.moveaxis(po.major45(po.neohookean_ddw(F, 1.3, 2.7)), 0, -1)
    for got, ref, what in ((w, z["neo_w"], "W"), (dw, z["neo_dw"], "DW"), (ddw, z["neo_ddw"], "DDW")):
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max(), what


def test_cubic_define_is_bitwise_the_reference(z):
    bitwise(models.cubic(1.68, 1.21, 0.75, z["cubic_R"]), z["cubic_tabs"], "Cubic::Define")


def test_fixtures_regenerate_from_the_reference_tree(z):
    from oracle.refshim import build_ref
    if not build_ref.available():
        pytest.skip("reference tree not present")
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_ref_golden", os.path.join(os.path.dirname(PATH), "make_ref_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    fresh = mod.make()
    assert sorted(fresh) == sorted(z.files)
    for k in z.files:
        assert np.array_equal(np.asarray(fresh[k]), z[k]), k
