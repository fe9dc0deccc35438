"""Host-side mirror of the reference's elasticity operator/solver interface over libaefast.

Same class and method names, argument meaning and error behaviour as
  Operator::Elastic<T>              src/Operator/Elastic.H:20-171
  BC::Operator::Elastic<T>          src/BC/Operator/Elastic.H:12-406
  Solver::Nonlocal::Linear          src/Solver/Nonlocal/Linear.H:19-143
  Solver::Nonlocal::Newton<T>       src/Solver/Nonlocal/Newton.H:15-349
with AMReX MultiFabs replaced by `Field` (one nodal patch per level, Array4 layout)
and Util::Abort replaced by AeError.  Every operation runs in libaefast.so on the GPU.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import AeError, Fab, LevelDesc, SolveStats, check, default_opts, load
from .models import DIAGONAL, ISOTROPIC, MAJOR, MAJORMINOR, NCOEF, NeoHookean

FACES = ["XLO", "YLO", "ZLO", "XHI", "YHI", "ZHI",
         "YLO_ZLO", "YLO_ZHI", "YHI_ZLO", "YHI_ZHI",
         "ZLO_XLO", "ZLO_XHI", "ZHI_XLO", "ZHI_XHI",
         "XLO_YLO", "XLO_YHI", "XHI_YLO", "XHI_YHI",
         "XLO_YLO_ZLO", "XLO_YLO_ZHI", "XLO_YHI_ZLO", "XLO_YHI_ZHI",
         "XHI_YLO_ZLO", "XHI_YLO_ZHI", "XHI_YHI_ZLO", "XHI_YHI_ZHI"]
FACE = {n: i for i, n in enumerate(FACES)}


class Field:
    """A nodal field over the index box [lo, lo + shape - 1]: array shaped (ncomp, nz, ny, nx),
    i fastest (AMReX Array4 order).  `arr` is a numpy array (host) or a torch tensor (device)."""

    def __init__(self, arr, lo=(0, 0, 0)):
        self.arr = arr
        self.lo = tuple(int(v) for v in lo)

    @property
    def hi(self):
        nz, ny, nx = self.arr.shape[1:]
        return (self.lo[0] + nx - 1, self.lo[1] + ny - 1, self.lo[2] + nz - 1)

    def fab(self):
        a = self.arr
        f = Fab()
        if isinstance(a, np.ndarray):
            if not a.flags.c_contiguous:
                raise ValueError("Field array must be C-contiguous")
            f.data = a.ctypes.data
            f.is_float = 1 if a.dtype == np.float32 else 0
        else:  # torch tensor
            if not a.is_contiguous():
                raise ValueError("Field tensor must be contiguous")
            f.data = a.data_ptr()
            f.is_float = 1 if str(a.dtype) == "torch.float32" else 0
        for d in range(3):
            f.lo[d] = self.lo[d]
            f.hi[d] = self.hi[d]
        f.ncomp = a.shape[0]
        return f


class BCElastic:
    """BC::Operator::Elastic<T>: a type and a value per face (26) and direction (3).
    Defaults to displacement 0 everywhere (src/BC/Operator/Elastic.H:46-55)."""
    Displacement, Traction, Periodic, Neumann = 0, 1, 2, 3
    X, Y, Z = 0, 1, 2
    _NAMES = {"displacement": 0, "disp": 0, "neumann": 3, "traction": 1, "trac": 1, "periodic": 2}

    def __init__(self):
        self.type = np.zeros((26, 3), dtype=np.int32)
        self.val = np.zeros((26, 3), dtype=np.float64)

    def Set(self, face, direction, type_, value):
        f = FACE[face] if isinstance(face, str) else int(face)
        self.type[f, direction] = type_
        self.val[f, direction] = value

    @staticmethod
    def Parse(value, pp):
        """Keys type.<face> = "disp trac neumann", val.<face> = "0 0 0.01", face names as in the
        reference input files (xlo, ylozlo, xhiyhizhi, ...) (src/BC/Operator/Elastic.H:318-405)."""
        for name, f in FACE.items():
            key = name.lower().replace("_", "")
            if "type." + key in pp:
                words = str(pp["type." + key]).split()
                for d in range(3):
                    value.type[f, d] = BCElastic._NAMES[words[d]]
            if "val." + key in pp:
                words = str(pp["val." + key]).split()
                for d in range(3):
                    value.val[f, d] = float(words[d])
        return value


def level_desc(domain_cells, lo=None, hi=None, dx=None):
    n = (domain_cells,) * 3 if np.isscalar(domain_cells) else tuple(domain_cells)
    L = LevelDesc()
    for d in range(3):
        L.domain_cells[d] = n[d]
        L.lo[d] = 0 if lo is None else lo[d]
        L.hi[d] = n[d] if hi is None else hi[d]
        L.dx[d] = (1.0 / n[d]) if dx is None else (dx if np.isscalar(dx) else dx[d])
    return L


class Elastic:
    """Operator::Elastic<T> over libaefast: one nodal patch per AMR level, multigrid
    levels built by coarsening AMR level 0 while possible."""

    def __init__(self, levels, model):
        lib = load()
        self.model = int(model)
        self.ncoef = NCOEF[self.model]
        arr = (LevelDesc * len(levels))(*levels)
        h = C.c_void_p()
        check(lib.ae_op_create(arr, len(levels), self.model, C.byref(h)))
        self._h = h
        self.levels = list(levels)
        self.m_bc = None

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().ae_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------- geometry
    def NAmrLevels(self):
        return load().ae_op_num_amr_levels(self._h)

    def NMGLevels(self, amrlev=0):
        return load().ae_op_num_mg_levels(self._h, amrlev)

    def level_info(self, amrlev=0, mglev=0):
        lo, hi, dh = (C.c_int * 3)(), (C.c_int * 3)(), (C.c_int * 3)()
        dx = (C.c_double * 3)()
        check(load().ae_op_level_info(self._h, amrlev, mglev, lo, hi, dh, dx))
        ng = 0 if amrlev == 0 else 2
        return tuple(lo), tuple(hi), tuple(dh), tuple(dx), ng

    def storage_box(self, amrlev=0, mglev=0):
        lo, hi, _, _, ng = self.level_info(amrlev, mglev)
        return tuple(v - ng for v in lo), tuple(v + ng for v in hi)

    # ------------------------------------------------------------- set-up
    def SetModel(self, a, coeffs=None):
        """SetModel(amrlev, Field) copies per-node coefficients; SetModel(coeffs) sets one
        stiffness on every node (src/Operator/Elastic.cpp:57-118)."""
        if coeffs is None:
            c = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
            check(load().ae_op_set_model_uniform(self._h, c.ctypes.data_as(C.POINTER(C.c_double)), c.size))
        else:
            f = coeffs.fab()
            check(load().ae_op_set_model(self._h, int(a), C.byref(f)))

    def SetModelGrains(self, a, grain_id, table):
        """SetModel(amrlev, ...) for a Voronoi stiffness: grain_id a Field of int32 ids (ncomp 1),
        table (ngrains, ncoef); equivalent to SetModel with C = table[grain_id]."""
        table = np.ascontiguousarray(table, dtype=np.float64)
        arr = grain_id.arr
        if isinstance(arr, np.ndarray):
            if arr.dtype != np.int32:
                raise TypeError("grain ids must be int32")
        elif str(arr.dtype) != "torch.int32":
            raise TypeError("grain ids must be int32")
        f = grain_id.fab()
        f.is_float = 0
        check(load().ae_op_set_model_grains(self._h, int(a), C.byref(f), table.shape[0], table.ctypes.data))

    def SetModelMixture(self, a, eta, table, F0table=None, F0=None):
        """SetModel(amrlev, ...) from cell-centred phase-field order parameters, mixed on the
        device as PhaseFieldMicrostructure::TimeStepBegin does with Affine::Cubic::Combine
        (src/Integrator/PhaseFieldMicrostructure.cpp:516-541, src/Model/Solid/Affine/Cubic.H:70-82).
        eta: a Field of FP64 cell values (nphase components) whose box is in cell indices;
        table (nphase, ncoef).  F0table (nphase, 9) and F0 (a 9-component nodal Field) go
        together: F0 receives the mixed eigenstrain."""
        if (F0table is None) != (F0 is None):
            raise ValueError("F0table and F0 go together")
        table = np.ascontiguousarray(table, dtype=np.float64)
        fe = eta.fab()
        f0t = None if F0table is None else np.ascontiguousarray(F0table, dtype=np.float64)
        ff = None if F0 is None else F0.fab()
        check(load().ae_op_set_model_mixture(self._h, int(a), C.byref(fe), table.shape[0], table.ctypes.data,
                                             None if f0t is None else f0t.ctypes.data,
                                             None if ff is None else C.addressof(ff)))

    def SetModelDegraded(self, a, eta, lambda0, mu0):
        """SetModel(amrlev, ...) for the isotropic degradable model, built on the device as
        PolymerDegradation::DegradeMaterial does (src/Integrator/PolymerDegradation.cpp:794-833):
        (lambda0, mu0) everywhere, (1 - e) times that on valid nodes, e the 8-cell mean of eta
        (a Field of FP64 cell values, box in cell indices; None for no degradation)."""
        if eta is None:
            check(load().ae_op_set_model_degraded(self._h, int(a), None, 0, float(lambda0), float(mu0)))
            return
        fe = eta.fab()
        check(load().ae_op_set_model_degraded(self._h, int(a), C.addressof(fe), fe.ncomp, float(lambda0),
                                              float(mu0)))

    def SetBC(self, bc):
        self.m_bc = bc
        t = np.ascontiguousarray(bc.type, dtype=np.int32)
        v = np.ascontiguousarray(bc.val, dtype=np.float64)
        check(load().ae_op_set_bc(self._h, t.ctypes.data_as(C.POINTER(C.c_int)),
                                  v.ctypes.data_as(C.POINTER(C.c_double))))

    def GetBC(self):
        return self.m_bc

    def SetUniform(self, uniform, homogeneous=False):
        self._uniform = bool(uniform)
        check(load().ae_op_set_flags(self._h, int(bool(uniform)), int(bool(homogeneous))))

    def SetHomogeneous(self, homogeneous):
        check(load().ae_op_set_flags(self._h, int(getattr(self, "_uniform", False)), int(bool(homogeneous))))

    def prepareForSolve(self):
        check(load().ae_op_prepare(self._h))

    def set_stream(self, stream_ptr):
        check(load().ae_op_set_stream(self._h, C.c_void_p(stream_ptr)))

    def device_bytes(self):
        return load().ae_op_device_bytes(self._h)

    # ------------------------------------------------------------- operator pieces (device Fields)
    def Fapply(self, amrlev, mglev, out, inp):
        fo, fi = out.fab(), inp.fab()
        check(load().ae_fapply(self._h, amrlev, mglev, C.byref(fo), C.byref(fi)))

    def Diagonal(self, amrlev, mglev, diag):
        f = diag.fab()
        check(load().ae_diagonal(self._h, amrlev, mglev, C.byref(f)))

    def Fsmooth(self, amrlev, mglev, x, b, nsweeps=2, omega=2.0 / 3.0):
        fx, fb = x.fab(), b.fab()
        check(load().ae_fsmooth(self._h, amrlev, mglev, C.byref(fx), C.byref(fb), int(nsweeps), float(omega)))

    def Residual(self, amrlev, mglev, r, x, b):
        fr, fx, fb = r.fab(), x.fab(), b.fab()
        n = C.c_double(0.0)
        check(load().ae_residual(self._h, amrlev, mglev, C.byref(fr), C.byref(fx), C.byref(fb), C.byref(n)))
        return n.value

    def restriction(self, amrlev, cmglev, crse, fine):
        fc, ff = crse.fab(), fine.fab()
        check(load().ae_restrict(self._h, amrlev, cmglev, C.byref(fc), C.byref(ff)))

    def interpolation(self, amrlev, fmglev, fine, crse):
        ff, fc = fine.fab(), crse.fab()
        check(load().ae_interp_add(self._h, amrlev, fmglev, C.byref(ff), C.byref(fc)))

    def BCInit(self, amrlev, rhs, homogeneous=False):
        """BC::Operator::Elastic<T>::Init(rhs, geom) for this operator's BC."""
        f = rhs.fab()
        check(load().ae_bc_init(self._h, amrlev, C.byref(f), int(bool(homogeneous))))

    def Strain(self, amrlev, eps, u, voigt=False):
        fe, fu = eps.fab(), u.fab()
        check(load().ae_strain(self._h, amrlev, C.byref(fe), C.byref(fu), int(bool(voigt))))

    def Stress(self, amrlev, sigma, u, voigt=False, homogeneous=False):
        fs, fu = sigma.fab(), u.fab()
        check(load().ae_stress(self._h, amrlev, C.byref(fs), C.byref(fu), int(bool(voigt))))

    def NewtonResidual(self, amrlev, rhs, u, b, F0=None):
        """rhs = b - N(u) (Newton<T>::prepareForSolve); device Fields."""
        fr, fu, fb = rhs.fab(), u.fab(), b.fab()
        f0 = F0.fab() if F0 is not None else None
        check(load().ae_newton_residual(self._h, amrlev, C.byref(fu), C.byref(fb),
                                        C.byref(f0) if f0 is not None else None, C.byref(fr)))

    def NewtonDW(self, amrlev, u, dw=None, w=None, F0=None):
        """Newton<T>::DW (9 components) and Newton<T>::W; device Fields."""
        fu = u.fab()
        fd = dw.fab() if dw is not None else None
        fw = w.fab() if w is not None else None
        f0 = F0.fab() if F0 is not None else None
        check(load().ae_newton_dw(self._h, amrlev, C.byref(fu), C.byref(f0) if f0 is not None else None,
                                  C.byref(fd) if fd is not None else None, C.byref(fw) if fw is not None else None))

    def NewtonNeoHookean(self, amrlev, rhs, u, b, model):
        """Newton<NeoHookean>::prepareForSolve on one level: the level's stiffness becomes
        DDW(I + grad u) and rhs = b - N(u) with DW(I + grad u) (ae_newton_neohookean).  The
        operator is of kind models.MAJOR; host or device Fields."""
        fr, fu, fb = rhs.fab(), u.fab(), b.fab()
        check(load().ae_newton_neohookean(self._h, amrlev, C.byref(fu), C.byref(fb), float(model.mu),
                                          float(model.kappa), C.byref(fr)))

    def NeoHookeanDW(self, amrlev, u, model, dw=None, w=None):
        """Newton<NeoHookean>::DW (9 components) and ::W at F = I + grad u; device Fields."""
        fu = u.fab()
        fd = dw.fab() if dw is not None else None
        fw = w.fab() if w is not None else None
        check(load().ae_neohookean_dw(self._h, amrlev, C.byref(fu), float(model.mu), float(model.kappa),
                                      C.byref(fd) if fd is not None else None,
                                      C.byref(fw) if fw is not None else None))

    def Energy(self, amrlev, energy, u, homogeneous=False):
        fw, fu = energy.fab(), u.fab()
        check(load().ae_energy(self._h, amrlev, C.byref(fw), C.byref(fu)))


class Linear:
    """Solver::Nonlocal::Linear: MLMG with the reference's defaults (bicgstab bottom,
    max_fmg_iter = 1e8, i.e. F-cycles) (src/Solver/Nonlocal/Linear.H:23-29)."""

    def __init__(self, op):
        self.linop = op
        self.opts = default_opts(max_fmg_iter=100000000, bottom=1, nu1=2, nu2=2)
        self.m_tol_rel = 1e-8
        self.m_tol_abs = 1e-8
        self.stats = SolveStats()

    def setMaxIter(self, n):
        self.opts.max_iter = int(n)

    def setBottomMaxIter(self, n):
        self.opts.bottom_max_iter = int(n)

    def setMaxFmgIter(self, n):
        self.opts.max_fmg_iter = int(min(n, 2 ** 31 - 1))

    def setFixedIter(self, n):
        """Run exactly n iterations, converged or not (MLMG fixed_iter)."""
        self.opts.fixed_iter = int(n)

    def setBottomSolver(self, name):
        self.opts.bottom = {"cg": 0, "bicgstab": 1}[name]

    def setPreSmooth(self, n):
        self.opts.nu1 = int(n)

    def setPostSmooth(self, n):
        self.opts.nu2 = int(n)

    def setVerbose(self, v):
        self.opts.verbose = int(v)

    def setPrecision(self, name):
        """'fp64' (plain drop-in) or 'mixed' (FP32 cycle inside FP64 refinement)."""
        self.opts.precision = {"fp64": 0, "mixed": 1}[name]

    def solve(self, sol, rhs, tol_rel=None, tol_abs=None):
        """MLMG::solve over one Field per AMR level (host numpy or device torch); returns the
        final residual max-norm."""
        sol = sol if isinstance(sol, (list, tuple)) else [sol]
        rhs = rhs if isinstance(rhs, (list, tuple)) else [rhs]
        fs = (Fab * len(sol))(*[s.fab() for s in sol])
        fr = (Fab * len(rhs))(*[r.fab() for r in rhs])
        tr = self.m_tol_rel if tol_rel is None else tol_rel
        ta = self.m_tol_abs if tol_abs is None else tol_abs
        check(load().ae_solve(self.linop.handle, fs, fr, float(tr), float(ta), C.byref(self.opts),
                              C.byref(self.stats)))
        return self.stats.resfinal

    def solveaffine(self, sol, rhs, tol_rel=None, tol_abs=None, copyrhs=False):
        """Linear::solveaffine (src/Solver/Nonlocal/Linear.H:41-100): rhs plus the negated apply of
        zero by the inhomogeneous operator (zero on the domain boundary), solved homogeneously;
        copyrhs writes that right-hand side back into rhs.  Returns the final residual max-norm."""
        sol = sol if isinstance(sol, (list, tuple)) else [sol]
        rhs = rhs if isinstance(rhs, (list, tuple)) else [rhs]
        fs = (Fab * len(sol))(*[s.fab() for s in sol])
        fr = (Fab * len(rhs))(*[r.fab() for r in rhs])
        tr = self.m_tol_rel if tol_rel is None else tol_rel
        ta = self.m_tol_abs if tol_abs is None else tol_abs
        check(load().ae_solveaffine(self.linop.handle, fs, fr, float(tr), float(ta), int(bool(copyrhs)),
                                    C.byref(self.opts), C.byref(self.stats)))
        return self.stats.resfinal

    @staticmethod
    def Parse(value, pp):
        """Keys of src/Solver/Nonlocal/Linear.H:121-140 plus bottom_solver, precision, pre/post smooth."""
        if "max_iter" in pp:
            value.setMaxIter(int(pp["max_iter"]))
        if "bottom_max_iter" in pp:
            value.setBottomMaxIter(int(pp["bottom_max_iter"]))
        if "max_fmg_iter" in pp:
            value.setMaxFmgIter(int(pp["max_fmg_iter"]))
        if "fixed_iter" in pp:
            value.setFixedIter(int(pp["fixed_iter"]))
        if "verbose" in pp:
            value.setVerbose(int(pp["verbose"]))
        if "bottom_solver" in pp:
            value.setBottomSolver(str(pp["bottom_solver"]))
        if "precision" in pp:
            value.setPrecision(str(pp["precision"]))
        if "pre_smooth" in pp:
            value.setPreSmooth(int(pp["pre_smooth"]))
        if "post_smooth" in pp:
            value.setPostSmooth(int(pp["post_smooth"]))
        if "tol_rel" in pp:
            value.m_tol_rel = float(pp["tol_rel"])
        if "tol_abs" in pp:
            value.m_tol_abs = float(pp["tol_abs"])
        return value


class Newton(Linear):
    """Solver::Nonlocal::Newton<T> (src/Solver/Nonlocal/Newton.H:141-205): m_nriters times,
    rhs = b - N(u), one Linear::solve of the correction (its previous value is the initial guess,
    as the reference keeps dsol), u += dsol.  For the linear and affine models the operator's
    stiffness is fixed and N(u) = div(C : (grad u - F0)) (ae_newton_residual; F0: per-level
    eigenstrain Fields, 9 components, of an Affine model, or None).  With model a
    models.NeoHookean the operator is of kind models.MAJOR and every iteration first sets its
    stiffness to the tangent DDW(I + grad u) and N(u) = div DW(I + grad u)
    (ae_newton_neohookean)."""

    def __init__(self, op):
        super().__init__(op)
        self.m_nriters = 1

    def setNRIters(self, n):
        self.m_nriters = int(n)

    @staticmethod
    def Parse(value, pp):
        """Newton<T>::Parse (src/Solver/Nonlocal/Newton.H:342-347): the Linear keys plus nriters."""
        Linear.Parse(value, pp)
        if "nriters" in pp:
            value.setNRIters(int(pp["nriters"]))
        return value

    def compResidual(self, res, u, b, F0=None):
        """Newton<T>::compResidual (src/Solver/Nonlocal/Newton.H:211-231): res = b - N(u) on every
        level (device Fields, one per level; F0 per-level eigenstrains or None)."""
        for lev in range(len(u)):
            self.linop.NewtonResidual(lev, res[lev], u[lev], b[lev], None if F0 is None else F0[lev])

    def W(self, w, u, F0=None, model=None):
        """Newton<T>::W (src/Solver/Nonlocal/Newton.H:233-275): strain energy density per node
        (model: a models.NeoHookean for the finite-kinematics W(I + grad u))."""
        for lev in range(len(u)):
            if isinstance(model, NeoHookean):
                self.linop.NeoHookeanDW(lev, u[lev], model, w=w[lev])
            else:
                self.linop.NewtonDW(lev, u[lev], w=w[lev], F0=None if F0 is None else F0[lev])

    def DW(self, dw, u, F0=None, model=None):
        """Newton<T>::DW (src/Solver/Nonlocal/Newton.H:277-333): DW, 9 components row-major
        (model: a models.NeoHookean for DW(I + grad u))."""
        for lev in range(len(u)):
            if isinstance(model, NeoHookean):
                self.linop.NeoHookeanDW(lev, u[lev], model, dw=dw[lev])
            else:
                self.linop.NewtonDW(lev, u[lev], dw=dw[lev], F0=None if F0 is None else F0[lev])

    def solve(self, u, b, model=None, tol_rel=None, tol_abs=None, F0=None):
        import torch
        u = u if isinstance(u, (list, tuple)) else [u]
        b = b if isinstance(b, (list, tuple)) else [b]
        F0 = [None] * len(u) if F0 is None else (F0 if isinstance(F0, (list, tuple)) else [F0])

        def dev(f):  # device copy of a host Field, or the Field itself
            if f is None or not isinstance(f.arr, np.ndarray):
                return f
            return Field(torch.from_numpy(np.ascontiguousarray(f.arr)).cuda(), f.lo)

        ud, bd, fd = [dev(f) for f in u], [dev(f) for f in b], [dev(f) for f in F0]
        dsol = [Field(torch.zeros_like(f.arr), f.lo) for f in ud]
        rhs = [Field(f.arr.clone(), f.lo) for f in bd]
        res = None
        for _ in range(self.m_nriters):
            for lev in range(len(ud)):
                if isinstance(model, NeoHookean):
                    self.linop.NewtonNeoHookean(lev, rhs[lev], ud[lev], bd[lev], model)
                    continue
                fu, fb, fr = ud[lev].fab(), bd[lev].fab(), rhs[lev].fab()
                f0 = fd[lev].fab() if fd[lev] is not None else None
                check(load().ae_newton_residual(self.linop.handle, lev, C.byref(fu), C.byref(fb),
                                                C.byref(f0) if f0 is not None else None, C.byref(fr)))
            res = Linear.solve(self, dsol, rhs, tol_rel, tol_abs)
            for lev in range(len(ud)):
                ud[lev].arr += dsol[lev].arr
        torch.cuda.synchronize()
        for f, g in zip(u, ud):
            if isinstance(f.arr, np.ndarray):
                f.arr[...] = g.arr.cpu().numpy()
        return res
