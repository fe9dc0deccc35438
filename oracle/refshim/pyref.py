"""ctypes access to oracle/_ref/libref.so: the reference's own per-node operator code compiled by
oracle/refshim/build_ref.py.  TEST INFRASTRUCTURE ONLY -- used to make and check golden vectors
(tests/golden/make_ref_golden.py); it needs the reference tree, so it runs only where that is
present.  Arguments follow the oracle's conventions (oracle/pyoracle.py): a level description
(pyoracle.Level), per-node coefficients [slot][k][j][i], fields [comp][k][j][i] over the level's
storage, BC tables (26, 3)."""
import ctypes as C

import numpy as np

from oracle import pyoracle as po

_lib = None


def lib():
    global _lib
    if _lib is None:
        from oracle.refshim import build_ref
        path = build_ref.build()
        if path is None:
            raise RuntimeError("the reference tree is not available: %s" % build_ref.reference_src())
        _lib = C.CDLL(path)
        _lib.ref_error.restype = C.c_char_p
    return _lib


def _slots():
    from anisotropicfracture_gb300 import models
    return np.ascontiguousarray(models.SLOT.reshape(-1).astype(np.int32))


def _d(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference code failed: %s" % lib().ref_error().decode())


def _bc(bctype, bcval):
    t, tp = _i(np.asarray(bctype).reshape(26, 3))
    v = np.ascontiguousarray(np.asarray(bcval, dtype=np.float64).reshape(26, 3)) if bcval is not None \
        else np.zeros((26, 3))
    return t, tp, v


def fapply(L, model, Cf, bctype, u, uniform=False, homogeneous=False, bcval=None):
    Cf, u = np.ascontiguousarray(Cf, dtype=np.float64), np.ascontiguousarray(u, dtype=np.float64)
    s, (t, tp, v) = _slots(), _bc(bctype, bcval)
    f = np.zeros_like(u)
    _check(lib().ref_fapply(C.byref(L), model, _d(Cf), _i(s)[1], tp, _d(v), int(uniform), int(homogeneous),
                            _d(u), _d(f)))
    return f


def diagonal(L, model, Cf, bctype, bcval=None):
    Cf = np.ascontiguousarray(Cf, dtype=np.float64)
    s, (t, tp, v) = _slots(), _bc(bctype, bcval)
    D = np.zeros((3,) + Cf.shape[1:])
    _check(lib().ref_diagonal(C.byref(L), model, _d(Cf), _i(s)[1], tp, _d(v), _d(D)))
    return D


def fsmooth(L, model, Cf, bctype, diag, x, b, uniform=False, bcval=None):
    """One reference Fsmooth call (two damped-Jacobi sweeps, omega = 2/3)."""
    Cf = np.ascontiguousarray(Cf, dtype=np.float64)
    diag, b = np.ascontiguousarray(diag, dtype=np.float64), np.ascontiguousarray(b, dtype=np.float64)
    x = np.array(x, dtype=np.float64, order="C")
    s, (t, tp, v) = _slots(), _bc(bctype, bcval)
    _check(lib().ref_fsmooth(C.byref(L), model, _d(Cf), _i(s)[1], tp, _d(v), int(uniform), _d(diag), _d(x), _d(b)))
    return x


def fields(L, model, Cf, which, u, voigt=False):
    """which: 'strain', 'stress' or 'energy'."""
    Cf, u = np.ascontiguousarray(Cf, dtype=np.float64), np.ascontiguousarray(u, dtype=np.float64)
    w = {"strain": 0, "stress": 1, "energy": 2}[which]
    nc = 1 if w == 2 else (6 if voigt else 9)
    out = np.zeros((nc,) + u.shape[1:])
    _check(lib().ref_fields(C.byref(L), model, _d(Cf), _i(_slots())[1], w, int(voigt), _d(u), _d(out)))
    return out


def average_down_coeffs(Lf, Lc, model, Cf):
    Cf = np.ascontiguousarray(Cf, dtype=np.float64)
    shape_c = tuple(Lc.hi[d] - Lc.lo[d] + 1 + 2 * Lc.ng for d in (2, 1, 0))
    Cc = np.zeros((Cf.shape[0],) + shape_c)
    _check(lib().ref_average_down_coeffs(C.byref(Lf), C.byref(Lc), model, _d(Cf), _i(_slots())[1], _d(Cc)))
    return Cc


def bc_init(L, bctype, bcval, rhs, homogeneous=False):
    rhs = np.array(rhs, dtype=np.float64, order="C")
    t, tp, v = _bc(bctype, bcval)
    _check(lib().ref_bc_init(C.byref(L), tp, _d(v), int(homogeneous), _d(rhs)))
    return rhs


def restrict(Lc, Lf, fine):
    fine = np.ascontiguousarray(fine, dtype=np.float64)
    shape_c = tuple(Lc.hi[d] - Lc.lo[d] + 1 + 2 * Lc.ng for d in (2, 1, 0))
    crse = np.zeros((fine.shape[0],) + shape_c)
    _check(lib().ref_restrict(C.byref(Lc), C.byref(Lf), fine.shape[0], _d(crse), _d(fine)))
    return crse


def interp_add(Lf, Lc, fine, crse):
    fine = np.array(fine, dtype=np.float64, order="C")
    crse = np.ascontiguousarray(crse, dtype=np.float64)
    _check(lib().ref_interp_add(C.byref(Lf), C.byref(Lc), fine.shape[0], _d(fine), _d(crse)))
    return fine


def cubic_define(C11, C12, C44, R):
    out = np.zeros(21)
    R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
    _check(lib().ref_cubic_define(C.c_double(C11), C.c_double(C12), C.c_double(C44), _d(R), _i(_slots())[1],
                                  _d(out)))
    return out


def level(*a, **k):
    return po.level(*a, **k)


def neohookean(mu, kappa, F):
    """Model::Solid::Elastic::NeoHookean W, DW and DDW of the reference at deformation gradients F
    (n, 3, 3): returns (w (n,), dw (n, 3, 3), ddw (n, 45) in the Sym::Major slot order)."""
    F = np.ascontiguousarray(np.asarray(F, dtype=np.float64).reshape(-1, 9))
    n = F.shape[0]
    w, dw, ddw = np.zeros(n), np.zeros((n, 9)), np.zeros((n, 45))
    _check(lib().ref_neohookean(C.c_double(mu), C.c_double(kappa), n, _d(F), _d(w), _d(dw), _d(ddw)))
    return w, dw.reshape(n, 3, 3), ddw
