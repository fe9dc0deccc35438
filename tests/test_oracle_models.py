"""The oracle's restatements of the two model-field builders the integrators run before their
elastic solve, checked against literal per-node restatements of the reference loops:
PhaseFieldMicrostructure::TimeStepBegin with Affine::Cubic::Combine
(src/Integrator/PhaseFieldMicrostructure.cpp:531-539, src/Model/Solid/Affine/Cubic.H:70-82) and
PolymerDegradation::DegradeMaterial with Degradable::Isotropic::DegradeModulus
(src/Integrator/PolymerDegradation.cpp:794-833, Degradable/Isotropic.H:74-81)."""
import numpy as np
import pytest

from oracle import pyoracle as po


def literal_mixture(lo, hi, eta, eta_lo, table, F0table):
    """One node at a time, as the reference's ParallelFor body and Combine do."""
    ncoef = table.shape[1]
    shape = tuple(hi[d] - lo[d] + 1 for d in (2, 1, 0))
    Cm = np.zeros((ncoef,) + shape)
    F0 = np.zeros((9,) + shape)

    def E(i, j, k, n):
        return eta[n, k - eta_lo[2], j - eta_lo[1], i - eta_lo[0]]

    for k in range(lo[2], hi[2] + 1):
        for j in range(lo[1], hi[1] + 1):
            for i in range(lo[0], hi[0] + 1):
                etas = [0.25 * (E(i, j, k, n) + E(i, j - 1, k, n) + E(i - 1, j, k, n) + E(i - 1, j - 1, k, n))
                        for n in range(eta.shape[0])]
                etasum = 0.0
                for n in range(len(etas)):
                    etasum += etas[n]
                ddw = [0.0] * ncoef
                f0 = [0.0] * 9
                for n in range(len(etas)):
                    for q in range(ncoef):
                        ddw[q] += table[n, q] * (etas[n] / etasum)
                    for r in range(9):
                        f0[r] += F0table[n, r] * (etas[n] / etasum)
                at = (k - lo[2], j - lo[1], i - lo[0])
                Cm[(slice(None),) + at] = ddw
                F0[(slice(None),) + at] = f0
    return Cm, F0


def literal_degraded(lo, hi, vlo, vhi, eta, eta_lo, lam0, mu0):
    shape = tuple(hi[d] - lo[d] + 1 for d in (2, 1, 0))
    Cm = np.empty((2,) + shape)
    Cm[0], Cm[1] = lam0, mu0

    def E(i, j, k, n):
        return eta[n, k - eta_lo[2], j - eta_lo[1], i - eta_lo[0]]

    mul = 1.0 / (2.0 + 2.0 + 4.0)
    for k in range(vlo[2], vhi[2] + 1):
        for j in range(vlo[1], vhi[1] + 1):
            for i in range(vlo[0], vhi[0] + 1):
                at = (k - lo[2], j - lo[1], i - lo[0])
                for n in range(eta.shape[0]):
                    temp = mul * (E(i, j, k, n) + E(i - 1, j, k, n) + E(i, j - 1, k, n) + E(i - 1, j - 1, k, n)
                                  + E(i, j, k - 1, n) + E(i - 1, j, k - 1, n) + E(i, j - 1, k - 1, n)
                                  + E(i - 1, j - 1, k - 1, n))
                    if temp < 0.0 or temp > 1.0:
                        raise ValueError("Invalid value of eta")
                    Cm[(0,) + at] = lam0 * (1.0 - temp)
                    Cm[(1,) + at] = mu0 * (1.0 - temp)
    return Cm


@pytest.mark.parametrize("ncoef", [2, 9, 21])
def test_mixture_restatement_matches_the_literal_loop(ncoef):
    rng = np.random.default_rng(ncoef)
    lo, hi = (-2, 1, 0), (3, 4, 6)
    nphase = 3
    eta_lo = (lo[0] - 1, lo[1] - 1, lo[2])
    eta = rng.random((nphase, hi[2] - lo[2] + 1, hi[1] - lo[1] + 2, hi[0] - lo[0] + 2))
    table = rng.standard_normal((nphase, ncoef))
    F0table = rng.standard_normal((nphase, 9))
    Cm, F0 = po.model_mixture(lo, hi, eta, eta_lo, table, F0table)
    Cl, Fl = literal_mixture(lo, hi, eta, eta_lo, table, F0table)
    assert np.array_equal(Cm, Cl) and np.array_equal(F0, Fl)


def test_mixture_of_one_phase_is_its_table():
    rng = np.random.default_rng(5)
    lo, hi = (0, 0, 0), (4, 4, 4)
    eta = 0.1 + rng.random((1, 5, 6, 6))
    table = rng.standard_normal((1, 21))
    Cm, _ = po.model_mixture(lo, hi, eta, (-1, -1, 0), table)
    assert np.allclose(Cm, table[0][:, None, None, None], rtol=1e-15, atol=0)


def test_cells_outside_eta_are_an_error():
    with pytest.raises(IndexError):
        po.model_degraded((0, 0, 0), (3, 3, 3), (0, 0, 0), (3, 3, 3), np.full((1, 4, 4, 4), 0.5), (-1, -1, -1), 1.0, 1.0)
    with pytest.raises(IndexError):
        po.model_mixture((0, 0, 0), (3, 3, 3), np.ones((1, 4, 5, 5)), (0, -1, 0), np.ones((1, 2)))


def test_mixture_zero_sum_gives_nan_as_the_reference_does():
    eta = np.zeros((2, 3, 4, 4))
    Cm, _ = po.model_mixture((0, 0, 0), (2, 2, 2), eta, (-1, -1, 0), np.ones((2, 2)))
    assert np.isnan(Cm).all()


def test_degraded_restatement_matches_the_literal_loop():
    rng = np.random.default_rng(11)
    lo, hi = (0, 0, 0), (7, 6, 5)
    vlo, vhi = (2, 2, 1), (5, 4, 4)
    eta_lo = tuple(v - 1 for v in vlo)
    eta = rng.random((2, vhi[2] - vlo[2] + 2, vhi[1] - vlo[1] + 2, vhi[0] - vlo[0] + 2))
    Cm = po.model_degraded(lo, hi, vlo, vhi, eta, eta_lo, 3.0, 1.5)
    assert np.array_equal(Cm, literal_degraded(lo, hi, vlo, vhi, eta, eta_lo, 3.0, 1.5))
    # the last component decides; nodes outside the valid box keep the undamaged values
    inner = (slice(1, 5), slice(2, 5), slice(2, 6))
    assert not np.array_equal(Cm[(0,) + inner], po.model_degraded(lo, hi, vlo, vhi, eta[:1], eta_lo, 3.0, 1.5)[(0,) + inner])
    assert np.all(Cm[0, 0] == 3.0) and np.all(Cm[1, :, :, 0] == 1.5)


def test_degraded_out_of_range_is_an_error():
    eta = np.full((1, 5, 5, 5), 0.5)
    eta[0, 1, 1, 1] = 9.0
    with pytest.raises(ValueError):
        po.model_degraded((0, 0, 0), (3, 3, 3), (0, 0, 0), (3, 3, 3), eta, (-1, -1, -1), 1.0, 1.0)
    with pytest.raises(ValueError):
        literal_degraded((0, 0, 0), (3, 3, 3), (0, 0, 0), (3, 3, 3), eta, (-1, -1, -1), 1.0, 1.0)
