"""ctypes front end of the CPU FP64 oracle (test infrastructure only).

Only tests/, the smoke check and bench.py's cpu_baseline leg import this module,
and only as the parity reference.  Fields are numpy float64 arrays shaped
(ncomp, nz, ny, nx) over the stored box grow(valid, ng), i fastest.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

ORC_ISOTROPIC, ORC_MAJORMINOR, ORC_DIAGONAL, ORC_MAJOR = 0, 1, 2, 3
NCOEF = {ORC_ISOTROPIC: 2, ORC_MAJORMINOR: 21, ORC_DIAGONAL: 9, ORC_MAJOR: 45}


class Level(C.Structure):
    _fields_ = [("dom_lo", C.c_int * 3), ("dom_hi", C.c_int * 3),
                ("lo", C.c_int * 3), ("hi", C.c_int * 3),
                ("ng", C.c_int), ("pad_", C.c_int), ("dx", C.c_double * 3)]

    @property
    def shape(self):
        return tuple(self.hi[d] - self.lo[d] + 1 + 2 * self.ng for d in (2, 1, 0))


class Opts(C.Structure):
    _fields_ = [("max_fmg_iter", C.c_int), ("nu1", C.c_int), ("nu2", C.c_int), ("sweeps", C.c_int),
                ("bottom", C.c_int), ("max_iter", C.c_int), ("bottom_max_iter", C.c_int),
                ("bottom_reltol", C.c_double), ("nuf", C.c_int), ("max_mg_levels", C.c_int),
                ("omega", C.c_double), ("uniform", C.c_int), ("pad_", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("iters", C.c_int), ("converged", C.c_int), ("nlevels", C.c_int),
                ("bottom_fail", C.c_int), ("res0", C.c_double), ("resfinal", C.c_double),
                ("target", C.c_double), ("hist", C.c_double * 256)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = C.CDLL(path)
        d = C.POINTER(C.c_double)
        i = C.POINTER(C.c_int)
        L = C.POINTER(Level)
        _lib.orc_fapply.argtypes = [L, C.c_int, d, i, C.c_int, d, d]
        _lib.orc_diagonal.argtypes = [L, C.c_int, d, i, d]
        _lib.orc_fsmooth.argtypes = [L, C.c_int, d, i, C.c_int, d, d, d, C.c_int, C.c_double]
        _lib.orc_residual.argtypes = [L, C.c_int, d, i, C.c_int, d, d, d, d]
        _lib.orc_restrict.argtypes = [L, L, C.c_int, d, d]
        _lib.orc_interp_add.argtypes = [L, L, C.c_int, d, d]
        _lib.orc_bc_init.argtypes = [L, i, d, C.c_int, d]
        _lib.orc_strain.argtypes = [L, d, C.c_int, d]
        _lib.orc_stress.argtypes = [L, C.c_int, d, d, C.c_int, d]
        _lib.orc_energy.argtypes = [L, C.c_int, d, d, d]
        _lib.orc_mm_full.argtypes = [d, d]
        _lib.orc_mm_stress.argtypes = [d, d, d]
        _lib.orc_mm_div.argtypes = [d, d, d]
        _lib.orc_solve.argtypes = [L, C.c_int, d, i, d, d, C.c_double, C.c_double,
                                   C.POINTER(Opts), C.POINTER(Stats)]
        _lib.orc_num_mg_levels.argtypes = [L, C.c_int]
        _lib.orc_set_threads.argtypes = [C.c_int]
    return _lib


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def level(n, dx=None, lo=(0, 0, 0), hi=None, ng=0, dom_hi=None):
    """Level over the nodal domain [0, n] per axis (n cells); valid box defaults to the domain."""
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    L = Level()
    dom_hi = n if dom_hi is None else dom_hi
    hi = dom_hi if hi is None else hi
    dx = tuple(1.0 / c for c in n) if dx is None else ((dx,) * 3 if np.isscalar(dx) else tuple(dx))
    for d in range(3):
        L.dom_lo[d] = 0
        L.dom_hi[d] = dom_hi[d]
        L.lo[d] = lo[d]
        L.hi[d] = hi[d]
        L.dx[d] = dx[d]
    L.ng = ng
    return L


def coarsen(L):
    Lc = Level()
    for d in range(3):
        Lc.dom_lo[d] = L.dom_lo[d] // 2
        Lc.dom_hi[d] = L.dom_hi[d] // 2
        Lc.lo[d] = L.lo[d] // 2
        Lc.hi[d] = L.hi[d] // 2
        Lc.dx[d] = L.dx[d] * 2.0
    Lc.ng = 0
    return Lc


def fapply(L, model, Cf, bctype, u, uniform=False):
    f = np.zeros_like(u)
    bt, bp = _i(bctype)
    lib().orc_fapply(C.byref(L), model, _d(Cf), bp, int(uniform), _d(u), _d(f))
    return f


def diagonal(L, model, Cf, bctype):
    D = np.zeros((3,) + L.shape)
    bt, bp = _i(bctype)
    lib().orc_diagonal(C.byref(L), model, _d(Cf), bp, _d(D))
    return D


def fsmooth(L, model, Cf, bctype, diag, x, b, nsweeps=2, omega=2.0 / 3.0, uniform=False):
    x = x.copy()
    bt, bp = _i(bctype)
    lib().orc_fsmooth(C.byref(L), model, _d(Cf), bp, int(uniform), _d(diag), _d(x), _d(b), nsweeps, omega)
    return x


def residual(L, model, Cf, bctype, x, b, uniform=False):
    r = np.zeros_like(x)
    nrm = C.c_double(0)
    bt, bp = _i(bctype)
    lib().orc_residual(C.byref(L), model, _d(Cf), bp, int(uniform), _d(x), _d(b), _d(r), C.byref(nrm))
    return r, nrm.value


def restrict(Lc, Lf, fine):
    ncomp = fine.shape[0]
    crse = np.zeros((ncomp,) + Lc.shape)
    lib().orc_restrict(C.byref(Lc), C.byref(Lf), ncomp, _d(crse), _d(np.ascontiguousarray(fine)))
    return crse


def interp_add(Lf, Lc, fine, crse):
    fine = fine.copy()
    lib().orc_interp_add(C.byref(Lf), C.byref(Lc), fine.shape[0], _d(fine), _d(np.ascontiguousarray(crse)))
    return fine


def bc_init(L, bctype, bcval, rhs, homogeneous=False):
    rhs = rhs.copy()
    bt, bp = _i(bctype)
    bv = np.ascontiguousarray(bcval, dtype=np.float64)
    lib().orc_bc_init(C.byref(L), bp, _d(bv), int(homogeneous), _d(rhs))
    return rhs


def strain(L, u, voigt=False):
    e = np.zeros((6 if voigt else 9,) + L.shape)
    lib().orc_strain(C.byref(L), _d(u), int(voigt), _d(e))
    return e


def stress(L, model, Cf, u, voigt=False):
    s = np.zeros((6 if voigt else 9,) + L.shape)
    lib().orc_stress(C.byref(L), model, _d(Cf), _d(u), int(voigt), _d(s))
    return s


def energy(L, model, Cf, u):
    w = np.zeros((1,) + L.shape)
    lib().orc_energy(C.byref(L), model, _d(Cf), _d(u), _d(w))
    return w


def mm_full(c21):
    out = np.zeros(81)
    lib().orc_mm_full(_d(np.ascontiguousarray(c21, dtype=np.float64)), _d(out))
    return out.reshape(3, 3, 3, 3)


def mm_stress(c21, g):
    s = np.zeros(9)
    lib().orc_mm_stress(_d(np.ascontiguousarray(c21, dtype=np.float64)),
                        _d(np.ascontiguousarray(g, dtype=np.float64).reshape(9)), _d(s))
    return s.reshape(3, 3)


def mm_div(c21, b):
    f = np.zeros(3)
    lib().orc_mm_div(_d(np.ascontiguousarray(c21, dtype=np.float64)),
                     _d(np.ascontiguousarray(b, dtype=np.float64).reshape(27)), _d(f))
    return f


def default_opts(**kw):
    o = Opts()
    o.max_fmg_iter, o.nu1, o.nu2, o.sweeps = 0, 1, 1, 2
    o.bottom, o.max_iter, o.bottom_max_iter = 0, 200, 200
    o.bottom_reltol, o.nuf, o.max_mg_levels = 1e-4, 8, 0
    o.omega, o.uniform = 2.0 / 3.0, 0
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def solve(L, model, Cf, bctype, u0, b, tol_rel=1e-8, tol_abs=0.0, **kw):
    u = u0.copy()
    o = default_opts(**kw)
    st = Stats()
    bt, bp = _i(bctype)
    rc = lib().orc_solve(C.byref(L), model, _d(Cf), bp, _d(u), _d(b), tol_rel, tol_abs, C.byref(o), C.byref(st))
    return u, st, rc


def num_mg_levels(L, max_mg_levels=0):
    return lib().orc_num_mg_levels(C.byref(L), max_mg_levels)


def set_threads(n):
    lib().orc_set_threads(int(n))


def solve_amr(Ls, model, Cs, bctype, us, bs, tol_rel=1e-8, tol_abs=0.0, **kw):
    """Composite solve over AMR levels; us are updated copies returned as a list."""
    n = len(Ls)
    lib().orc_solve_amr.argtypes = [C.POINTER(Level), C.c_int, C.c_int, C.POINTER(C.POINTER(C.c_double)),
                                    C.POINTER(C.c_int), C.POINTER(C.POINTER(C.c_double)),
                                    C.POINTER(C.POINTER(C.c_double)), C.c_double, C.c_double,
                                    C.POINTER(Opts), C.POINTER(Stats)]
    La = (Level * n)(*Ls)
    us = [u.copy() for u in us]
    Cs = [np.ascontiguousarray(c) for c in Cs]
    bs = [np.ascontiguousarray(b) for b in bs]
    Cp = (C.POINTER(C.c_double) * n)(*[_d(c) for c in Cs])
    up = (C.POINTER(C.c_double) * n)(*[_d(u) for u in us])
    bp = (C.POINTER(C.c_double) * n)(*[_d(b) for b in bs])
    o = default_opts(**kw)
    st = Stats()
    bt, btp = _i(bctype)
    rc = lib().orc_solve_amr(La, n, model, Cp, btp, up, bp, tol_rel, tol_abs, C.byref(o), C.byref(st))
    return us, st, rc


def residual_amr(Ls, model, Cs, bctype, us, bs, uniform=False, want_fields=False):
    """Composite residual max-norm of the solutions `us` (MLMG::computeMLResidual restated:
    per-level b - A u, reflux of each finer level's residual onto the coarse nodes it covers).
    Returns the norm, or (norm, per-level residual fields) with want_fields."""
    n = len(Ls)
    f = lib().orc_residual_amr
    f.argtypes = [C.POINTER(Level), C.c_int, C.c_int, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int),
                  C.c_int, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.POINTER(C.c_double)),
                  C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_double)]
    La = (Level * n)(*Ls)
    Cs = [np.ascontiguousarray(c, dtype=np.float64) for c in Cs]
    us = [np.ascontiguousarray(u, dtype=np.float64) for u in us]
    bs = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
    rs = [np.zeros_like(u) for u in us] if want_fields else None
    Cp = (C.POINTER(C.c_double) * n)(*[_d(c) for c in Cs])
    up = (C.POINTER(C.c_double) * n)(*[_d(u) for u in us])
    bp = (C.POINTER(C.c_double) * n)(*[_d(b) for b in bs])
    rp = (C.POINTER(C.c_double) * n)(*[_d(r) for r in rs]) if want_fields else None
    bt, btp = _i(bctype)
    nrm = C.c_double(0.0)
    rc = f(La, n, model, Cp, btp, int(uniform), up, bp, rp, C.byref(nrm))
    if rc != 0:
        raise RuntimeError("orc_residual_amr failed: %d" % rc)
    return (nrm.value, rs) if want_fields else nrm.value


def amr_levels(n, nlev, shrink=4):
    """Levels of the reference's test hierarchy (src/Test/Operator/Elastic.cpp:59-92): level 0
    n^3 cells on the unit cube; each finer level refines the central half of the previous one."""
    Ls = [level(n)]
    lo, hi = 0, n  # cell box of the previous level's patch, its own index space
    for l in range(1, nlev):
        cells = n * 2 ** l
        clo, chi = lo + (hi - lo) // shrink, hi - (hi - lo) // shrink
        lo, hi = 2 * clo, 2 * chi
        Ls.append(level(cells, lo=(lo,) * 3, hi=(hi,) * 3, ng=2))
    return Ls


def node_coords(L):
    """x, y, z of every stored node of a level (arrays shaped like one component)."""
    ax = [(np.arange(L.lo[d] - L.ng, L.hi[d] + L.ng + 1)) * L.dx[d] for d in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return X, Y, Z


# ---------------------------------------------------------------- Newton pieces
def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def newton_residual(L, model, Cf, bctype, u, b, F0=None, rhs=None):
    """rhs = b - N(u) on grow(valid, 1) ∩ domain (other nodes keep rhs, default b)."""
    lb = lib()
    d = C.POINTER(C.c_double)
    lb.orc_newton_residual.argtypes = [C.POINTER(Level), C.c_int, d, C.POINTER(C.c_int), d, d, d, d]
    out = np.array(b, dtype=np.float64, copy=True) if rhs is None else np.array(rhs, dtype=np.float64, copy=True)
    Cf, u, b, F0 = _f64(Cf), _f64(u), _f64(b), _f64(F0)  # kept alive across the call
    bt, bp = _i(bctype)
    lb.orc_newton_residual(C.byref(L), model, _d(Cf), bp, _d(u), _d(b), None if F0 is None else _d(F0), _d(out))
    return out


def newton_dw(L, model, Cf, u, F0=None):
    """(dw: 9 x shape, w: shape) on the valid box."""
    lb = lib()
    d = C.POINTER(C.c_double)
    lb.orc_newton_dw.argtypes = [C.POINTER(Level), C.c_int, d, d, d, d, d]
    dw = np.zeros((9,) + L.shape)
    w = np.zeros(L.shape)
    Cf, u, F0 = _f64(Cf), _f64(u), _f64(F0)
    lb.orc_newton_dw(C.byref(L), model, _d(Cf), _d(u), None if F0 is None else _d(F0), _d(dw), _d(w))
    return dw, w


def newton_grad(L, u):
    """grad u (9 components, row-major) on grow(valid, 2) ∩ domain with Newton::prepareForSolve's
    stencils (src/Solver/Nonlocal/Newton.H:52-58); zero elsewhere."""
    lb = lib()
    d = C.POINTER(C.c_double)
    lb.orc_newton_grad.argtypes = [C.POINTER(Level), d, d]
    g = np.zeros((9,) + L.shape)
    u = _f64(u)
    lb.orc_newton_grad(C.byref(L), _d(u), _d(g))
    return g


def newton_residual_dw(L, bctype, u, b, dw, rhs=None):
    """rhs = b - N(u) from a DW field the caller evaluated (9 components over the storage box),
    as Newton::prepareForSolve forms it (src/Solver/Nonlocal/Newton.H:84-136)."""
    lb = lib()
    d = C.POINTER(C.c_double)
    lb.orc_newton_residual_dw.argtypes = [C.POINTER(Level), C.POINTER(C.c_int), d, d, d, d]
    out = np.array(b if rhs is None else rhs, dtype=np.float64, copy=True)
    u, b, dw = _f64(u), _f64(b), _f64(dw)
    bt, bp = _i(bctype)
    lb.orc_newton_residual_dw(C.byref(L), bp, _d(u), _d(b), _d(dw), _d(out))
    return out


def neohookean_newton_residual(L, mu, kappa, bctype, u, b):
    """Newton::prepareForSolve for Model::Solid::Elastic::NeoHookean (kinematic variable F,
    Newton.H:70-75): dw = DW(I + grad u) node by node, then rhs = b - N(u).  Also returns the
    tangent DDW(I + grad u) per node, shaped (nz, ny, nx, 3, 3, 3, 3)."""
    g = newton_grad(L, u)
    F = np.moveaxis(g, 0, -1).reshape(L.shape + (3, 3)) + np.eye(3)
    dw = np.ascontiguousarray(np.moveaxis(neohookean_dw(F, mu, kappa).reshape(L.shape + (9,)), -1, 0))
    return newton_residual_dw(L, bctype, u, b, dw), neohookean_ddw(F, mu, kappa)


# ---------------------------------------------------------------- NeoHookean (finite kinematics)
def _neo_parts(F):
    F = np.asarray(F, dtype=np.float64)
    J = np.linalg.det(F)
    J23 = np.abs(J) ** (2.0 / 3.0)
    tr = np.einsum("...ij,...ij->...", F, F)  # trace(F F^T)
    FinvT = np.swapaxes(np.linalg.inv(F), -1, -2)
    return F, J, J23, tr, FinvT


def neohookean_w(F, mu, kappa):
    """Model::Solid::Elastic::NeoHookean::W (src/Model/Solid/Elastic/NeoHookean.H:19-27):
    mu/2 (tr(F F^T) / |J|^(2/3) - 3) + kappa/2 (J - 1)^2.  F: (..., 3, 3)."""
    F, J, J23, tr, _ = _neo_parts(F)
    return 0.5 * mu * (tr / J23 - 3.0) + 0.5 * kappa * (J - 1.0) * (J - 1.0)


def neohookean_dw(F, mu, kappa):
    """NeoHookean::DW (NeoHookean.H:28-39): mu (F / J23 - tr F^-T / (3 J23)) + kappa (J - 1) J F^-T."""
    F, J, J23, tr, FinvT = _neo_parts(F)
    J23, tr, J = J23[..., None, None], tr[..., None, None], J[..., None, None]
    return mu * (F / J23 - tr * FinvT / (3.0 * J23)) + kappa * (J - 1.0) * J * FinvT


def neohookean_ddw(F, mu, kappa):
    """NeoHookean::DDW (NeoHookean.H:40-66), the Sym::Major tangent ddw[..., i, j, k, l]:
    (mu / J23) t1 + kappa J t2 with
    t1 = d_ik d_jl - 2/3 F_ij G_kl - 2/3 G_ij F_kl + 2/9 tr G_ij G_kl + 1/3 tr G_il G_kj,
    t2 = (2J - 1) G_ij G_kl + (1 - J) G_il G_kj,  G = F^-T."""
    F, J, J23, tr, G = _neo_parts(F)
    I = np.eye(3)
    d = np.einsum("ik,jl->ijkl", I, I)
    t1 = (d - (2.0 / 3.0) * np.einsum("...ij,...kl->...ijkl", F, G)
          - (2.0 / 3.0) * np.einsum("...ij,...kl->...ijkl", G, F)
          + (2.0 / 9.0) * tr[..., None, None, None, None] * np.einsum("...ij,...kl->...ijkl", G, G)
          + (1.0 / 3.0) * tr[..., None, None, None, None] * np.einsum("...il,...kj->...ijkl", G, G))
    Jb = J[..., None, None, None, None]
    t2 = ((2.0 * Jb - 1.0) * np.einsum("...ij,...kl->...ijkl", G, G)
          + (1.0 - Jb) * np.einsum("...il,...kj->...ijkl", G, G))
    return (mu / J23[..., None, None, None, None]) * t1 + kappa * Jb * t2


def major45(ddw):
    """Set::Matrix4<3, Sym::Major> storage (src/Set/Matrix4_Major.H:203-258) of tensors shaped
    (..., 3, 3, 3, 3): slot s of the upper triangle (I, K), I <= K, of the 9 x 9 matrix
    A(3i+j, 3k+l), row by row; returned as (45, ...) per-node coefficient fields.  A slot holds
    the entry (K, I) below the diagonal: NeoHookean::DDW (NeoHookean.H:44-63) assigns both
    entries of a pair through the one slot in (i, j, k, l) order, so the lower one is written
    last and kept (the tensor is major-symmetric up to rounding)."""
    ddw = np.asarray(ddw, dtype=np.float64)
    A = ddw.reshape(ddw.shape[:-4] + (9, 9))
    rows, cols = np.triu_indices(9)
    return np.ascontiguousarray(np.moveaxis(A[..., cols, rows], -1, 0))


def neohookean_newton(L, mu, kappa, bctype, u, b, nriters=6, tol_rel=1e-10, tol_abs=0.0, **kw):
    """Solver::Nonlocal::Newton<NeoHookean>::solve restated (src/Solver/Nonlocal/Newton.H:142-209):
    each iteration forms rhs = b - N(u) and the tangent DDW(I + grad u) node by node
    (prepareForSolve), solves the tangent operator for the correction starting from the previous
    correction (the reference never resets it), and adds it to u.  Returns (u, [max |correction|
    per iteration])."""
    u = np.array(u, dtype=np.float64, copy=True)
    du = np.zeros_like(u)
    hist = []
    for _ in range(nriters):
        rhs, ddw = neohookean_newton_residual(L, mu, kappa, bctype, u, b)
        C = major45(ddw)
        du, st, rc = solve(L, ORC_MAJOR, C, bctype, du, rhs, tol_rel, tol_abs, **kw)
        if rc != 0:
            raise RuntimeError("tangent solve did not converge")
        hist.append(float(np.abs(du).max()))
        u += du
    return u, hist


# ---------------------------------------------------------------- stiffness from order parameters
def _cells(eta, eta_lo, lo, hi, di, dj, dk):
    """eta over the nodal box [lo, hi] shifted by (di, dj, dk) cells: the array of
    eta(i + di, j + dj, k + dk) for every node (i, j, k) of the box, all components."""
    sl = tuple(slice(lo[d] + s - eta_lo[d], hi[d] + s - eta_lo[d] + 1) for d, s in ((2, dk), (1, dj), (0, di)))
    for a, q in enumerate(sl):
        if q.start < 0 or q.stop > eta.shape[1 + a]:
            raise IndexError("eta does not cover the cells the nodes read")
    return eta[(slice(None),) + sl]


def model_mixture(lo, hi, eta, eta_lo, table, F0table=None):
    """The phase-field model field restated (src/Integrator/PhaseFieldMicrostructure.cpp:531-539
    with Affine::Cubic::Combine, src/Model/Solid/Affine/Cubic.H:70-82) over the nodal box
    [lo, hi]: e_n = 0.25 (eta_n(i,j,k) + eta_n(i,j-1,k) + eta_n(i-1,j,k) + eta_n(i-1,j-1,k)),
    C = sum_n table[n] (e_n / sum_m e_m), summed from zero in phase order, and F0 likewise.
    eta: (nphase, cz, cy, cx) cell values whose first cell is eta_lo.  Where the e_n sum to zero
    the reference divides by zero, and so does this (NaN)."""
    table = np.asarray(table, dtype=np.float64)
    e = 0.25 * (_cells(eta, eta_lo, lo, hi, 0, 0, 0) + _cells(eta, eta_lo, lo, hi, 0, -1, 0)
                + _cells(eta, eta_lo, lo, hi, -1, 0, 0) + _cells(eta, eta_lo, lo, hi, -1, -1, 0))
    s = np.zeros(e.shape[1:])
    for n in range(e.shape[0]):
        s = s + e[n]
    with np.errstate(invalid="ignore", divide="ignore"):
        w = e / s[None]
    Cm = np.zeros((table.shape[1],) + e.shape[1:])
    for n in range(e.shape[0]):
        Cm = Cm + table[n][:, None, None, None] * w[n][None]
    F0 = None
    if F0table is not None:
        F0table = np.asarray(F0table, dtype=np.float64)
        F0 = np.zeros((9,) + e.shape[1:])
        for n in range(e.shape[0]):
            F0 = F0 + F0table[n][:, None, None, None] * w[n][None]
    return Cm, F0


def model_degraded(lo, hi, vlo, vhi, eta, eta_lo, lambda0, mu0):
    """The degradable isotropic model field restated (src/Integrator/PolymerDegradation.cpp:794-833,
    src/Model/Solid/LinearElastic/Degradable/Isotropic.H:74-81) over the nodal box [lo, hi]:
    (lambda0, mu0) everywhere; on the valid nodes [vlo, vhi], for each component in turn,
    e = (1/8) times the sum of its 8 cells around the node (the reference's order) checked to lie
    in [0, 1] (ValueError otherwise, where the reference aborts), the last one kept:
    (lambda0 (1 - e), mu0 (1 - e))."""
    shape = tuple(hi[d] - lo[d] + 1 for d in (2, 1, 0))
    Cm = np.empty((2,) + shape)
    Cm[0], Cm[1] = lambda0, mu0
    if eta is None or eta.shape[0] == 0:
        return Cm
    c = lambda di, dj, dk: _cells(eta, eta_lo, vlo, vhi, di, dj, dk)
    e = 0.125 * (c(0, 0, 0) + c(-1, 0, 0) + c(0, -1, 0) + c(-1, -1, 0)
                 + c(0, 0, -1) + c(-1, 0, -1) + c(0, -1, -1) + c(-1, -1, -1))
    for n in range(e.shape[0]):
        if not np.all((e[n] >= 0.0) & (e[n] <= 1.0)):
            raise ValueError("Invalid value of eta")
    v = tuple(slice(vlo[d] - lo[d], vhi[d] - lo[d] + 1) for d in (2, 1, 0))
    Cm[(0,) + v] = lambda0 * (1.0 - e[-1])
    Cm[(1,) + v] = mu0 * (1.0 - e[-1])
    return Cm


# ---------------------------------------------------------------- periodic cells
class RveLevel(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("pad_", C.c_int), ("dx", C.c_double * 3)]

    @property
    def shape(self):
        return (self.n[2], self.n[1], self.n[0])


def _rve_lib():
    lb = lib()
    if not getattr(lb, "_rve_ready", False):
        d = C.POINTER(C.c_double)
        R = C.POINTER(RveLevel)
        lb.orc_rve_num_mg_levels.argtypes = [R, C.c_int]
        lb.orc_rve_fapply.argtypes = [R, C.c_int, d, C.c_int, d, d]
        lb.orc_rve_diagonal.argtypes = [R, C.c_int, d, d]
        lb.orc_rve_fsmooth.argtypes = [R, C.c_int, d, C.c_int, d, d, d, C.c_int, C.c_double]
        lb.orc_rve_residual.argtypes = [R, C.c_int, d, C.c_int, d, d, d, C.c_int, d, d]
        lb.orc_rve_restrict.argtypes = [R, R, C.c_int, d, d]
        lb.orc_rve_interp_add.argtypes = [R, R, C.c_int, d, d]
        lb.orc_rve_rhs.argtypes = [R, C.c_int, d, C.c_int, d, d]
        lb.orc_rve_mean_stress.argtypes = [R, C.c_int, d, d, d, d]
        lb.orc_rve_solve.argtypes = [R, C.c_int, d, d, d, C.c_double, C.c_double, C.POINTER(Opts),
                                     C.POINTER(Stats), d]
        lb._rve_ready = True
    return lb


def rve_level(n, length=1.0):
    """Periodic cell of n (int or 3 ints) cells per side on a cube of edge `length`."""
    n = (n,) * 3 if np.isscalar(n) else tuple(n)
    L = RveLevel()
    for d in range(3):
        L.n[d] = n[d]
        L.dx[d] = length / n[d]
    return L


def rve_coarsen(L):
    Lc = RveLevel()
    for d in range(3):
        Lc.n[d] = L.n[d] // 2
        Lc.dx[d] = 2.0 * L.dx[d]
    return Lc


def rve_num_mg_levels(L, max_mg_levels=0):
    return _rve_lib().orc_rve_num_mg_levels(C.byref(L), max_mg_levels)


def rve_fapply(L, model, Cf, u, uniform=False):
    f = np.zeros((3,) + L.shape)
    _rve_lib().orc_rve_fapply(C.byref(L), model, _d(Cf), int(uniform), _d(np.ascontiguousarray(u)), _d(f))
    return f


def rve_diagonal(L, model, Cf):
    D = np.zeros((3,) + L.shape)
    _rve_lib().orc_rve_diagonal(C.byref(L), model, _d(Cf), _d(D))
    return D


def rve_fsmooth(L, model, Cf, diag, x, b, nsweeps=2, omega=2.0 / 3.0, uniform=False):
    x = x.copy()
    _rve_lib().orc_rve_fsmooth(C.byref(L), model, _d(Cf), int(uniform), _d(diag), _d(x), _d(b), nsweeps, omega)
    return x


def rve_residual(L, model, Cf, x, b, project=True, uniform=False):
    r = np.zeros((3,) + L.shape)
    mean = np.zeros(3)
    nrm = C.c_double()
    _rve_lib().orc_rve_residual(C.byref(L), model, _d(Cf), int(uniform), _d(x), _d(b), _d(r), int(project),
                                _d(mean), C.cast(C.byref(nrm), C.POINTER(C.c_double)))
    return r, mean, nrm.value


def rve_restrict(Lc, Lf, fine):
    ncomp = fine.shape[0]
    c = np.zeros((ncomp,) + Lc.shape)
    assert _rve_lib().orc_rve_restrict(C.byref(Lc), C.byref(Lf), ncomp, _d(c), _d(np.ascontiguousarray(fine))) == 0
    return c


def rve_interp_add(Lf, Lc, fine, crse):
    fine = fine.copy()
    assert _rve_lib().orc_rve_interp_add(C.byref(Lf), C.byref(Lc), fine.shape[0], _d(fine),
                                         _d(np.ascontiguousarray(crse))) == 0
    return fine


def rve_rhs(L, model, Cf, E, uniform=False):
    b = np.zeros((3,) + L.shape)
    _rve_lib().orc_rve_rhs(C.byref(L), model, _d(Cf), int(uniform),
                           _d(np.ascontiguousarray(E, dtype=np.float64).reshape(9)), _d(b))
    return b


def rve_mean_stress(L, model, Cf, E, w):
    s = np.zeros(9)
    _rve_lib().orc_rve_mean_stress(C.byref(L), model, _d(Cf), _d(np.ascontiguousarray(E, dtype=np.float64).reshape(9)),
                                   _d(np.ascontiguousarray(w)), _d(s))
    return s.reshape(3, 3)


def rve_solve(L, model, Cf, E, w0=None, tol_rel=1e-8, tol_abs=0.0, **kw):
    """Periodic cell solve; returns (w with zero mean, stats, rc, body force)."""
    w = np.zeros((3,) + L.shape) if w0 is None else w0.copy()
    o = default_opts(**kw)
    st = Stats()
    bf = np.zeros(3)
    rc = _rve_lib().orc_rve_solve(C.byref(L), model, _d(Cf), _d(np.ascontiguousarray(E, dtype=np.float64).reshape(9)),
                                  _d(w), tol_rel, tol_abs, C.byref(o), C.byref(st), _d(bf))
    return w, st, rc, bf
