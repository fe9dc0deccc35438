"""ctypes binding of libaefast.so (include/aefast.h).

The library is the product: there is no CPU fallback.  Loading fails loudly when
the shared object has not been built (anisotropicfracture_gb300.build.build()).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libaefast.so")

AE_OK, AE_ERR_ARG, AE_ERR_NAN, AE_ERR_NOT_CONVERGED, AE_ERR_OOM, AE_ERR_CUDA, AE_ERR_STATE = 0, -1, -2, -3, -4, -5, -6
STATUS_NAMES = {0: "AE_OK", -1: "AE_ERR_ARG", -2: "AE_ERR_NAN", -3: "AE_ERR_NOT_CONVERGED",
                -4: "AE_ERR_OOM", -5: "AE_ERR_CUDA", -6: "AE_ERR_STATE"}


class AeError(RuntimeError):
    """Raised for a nonzero ae_status; mirrors Util::Abort, which throws in the reference."""

    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, code), msg))
        self.code = code


class LevelDesc(C.Structure):
    _fields_ = [("domain_cells", C.c_int * 3), ("lo", C.c_int * 3), ("hi", C.c_int * 3), ("dx", C.c_double * 3)]


class Fab(C.Structure):
    _fields_ = [("data", C.c_void_p), ("lo", C.c_int * 3), ("hi", C.c_int * 3), ("ncomp", C.c_int),
                ("is_float", C.c_int)]


class SolverOpts(C.Structure):
    _fields_ = [("max_fmg_iter", C.c_int), ("nu1", C.c_int), ("nu2", C.c_int), ("sweeps", C.c_int), ("bottom", C.c_int),
                ("max_iter", C.c_int), ("bottom_max_iter", C.c_int), ("bottom_reltol", C.c_double),
                ("nuf", C.c_int), ("max_mg_levels", C.c_int), ("omega", C.c_double), ("precision", C.c_int),
                ("inner_cycles", C.c_int), ("verbose", C.c_int), ("use_graph", C.c_int), ("fixed_iter", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iters", C.c_int), ("cycles", C.c_int), ("converged", C.c_int), ("nlevels", C.c_int),
                ("bottom_fail", C.c_int), ("pad_", C.c_int), ("res0", C.c_double), ("resfinal", C.c_double),
                ("target", C.c_double), ("seconds", C.c_double)]


class CellDesc(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("nrhs", C.c_int), ("length", C.c_double * 3)]


class CellStats(C.Structure):
    _fields_ = [("iters", C.c_int), ("converged", C.c_int), ("nlevels", C.c_int), ("bottom_fail", C.c_int),
                ("res0", C.c_double), ("resfinal", C.c_double), ("target", C.c_double), ("seconds", C.c_double),
                ("body_force", C.c_double * 3), ("mean_stress", C.c_double * 9)]


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_longlong), ("max_live_solves", C.c_int), ("keep_solution", C.c_int),
                ("tol_rel", C.c_double), ("tol_abs", C.c_double), ("solver", SolverOpts)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("nrhs", C.c_int), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("latency", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("queued", C.c_longlong), ("iterations", C.c_longlong), ("hbm_used", C.c_longlong),
                ("hbm_budget", C.c_longlong), ("busy_seconds", C.c_double), ("uptime_seconds", C.c_double)]


# (name, argtypes) of every exported entry point; include/aefast.h declares the same set
P = C.c_void_p
FAB = C.POINTER(Fab)
DP = C.POINTER(C.c_double)
SIGNATURES = {
    "ae_last_error": ([], C.c_char_p),
    "ae_version": ([], C.c_char_p),
    "ae_default_solver_opts": ([C.POINTER(SolverOpts)], None),
    "ae_op_create": ([C.POINTER(LevelDesc), C.c_int, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "ae_op_destroy": ([P], C.c_int),
    "ae_op_set_stream": ([P, P], C.c_int),
    "ae_op_set_model": ([P, C.c_int, FAB], C.c_int),
    "ae_op_set_model_uniform": ([P, C.POINTER(C.c_double), C.c_int], C.c_int),
    "ae_op_set_model_grains": ([P, C.c_int, FAB, C.c_int, C.c_void_p], C.c_int),
    "ae_op_set_model_mixture": ([P, C.c_int, FAB, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ae_op_set_model_degraded": ([P, C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double], C.c_int),
    "ae_op_set_bc": ([P, C.POINTER(C.c_int), C.POINTER(C.c_double)], C.c_int),
    "ae_op_set_flags": ([P, C.c_int, C.c_int], C.c_int),
    "ae_op_prepare": ([P], C.c_int),
    "ae_op_num_amr_levels": ([P], C.c_int),
    "ae_op_num_mg_levels": ([P, C.c_int], C.c_int),
    "ae_op_level_info": ([P, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                          C.POINTER(C.c_double)], C.c_int),
    "ae_op_device_bytes": ([P], C.c_longlong),
    "ae_fapply": ([P, C.c_int, C.c_int, FAB, FAB], C.c_int),
    "ae_diagonal": ([P, C.c_int, C.c_int, FAB], C.c_int),
    "ae_fsmooth": ([P, C.c_int, C.c_int, FAB, FAB, C.c_int, C.c_double], C.c_int),
    "ae_residual": ([P, C.c_int, C.c_int, FAB, FAB, FAB, C.POINTER(C.c_double)], C.c_int),
    "ae_restrict": ([P, C.c_int, C.c_int, FAB, FAB], C.c_int),
    "ae_interp_add": ([P, C.c_int, C.c_int, FAB, FAB], C.c_int),
    "ae_bc_init": ([P, C.c_int, FAB, C.c_int], C.c_int),
    "ae_strain": ([P, C.c_int, FAB, FAB, C.c_int], C.c_int),
    "ae_stress": ([P, C.c_int, FAB, FAB, C.c_int], C.c_int),
    "ae_energy": ([P, C.c_int, FAB, FAB], C.c_int),
    "ae_newton_residual": ([P, C.c_int, FAB, FAB, FAB, FAB], C.c_int),
    "ae_newton_dw": ([P, C.c_int, FAB, FAB, FAB, FAB], C.c_int),
    "ae_newton_neohookean": ([P, C.c_int, FAB, FAB, C.c_double, C.c_double, FAB], C.c_int),
    "ae_neohookean_dw": ([P, C.c_int, FAB, C.c_double, C.c_double, FAB, FAB], C.c_int),
    "ae_solve": ([P, FAB, FAB, C.c_double, C.c_double, C.POINTER(SolverOpts), C.POINTER(SolveStats)], C.c_int),
    "ae_solveaffine": ([P, FAB, FAB, C.c_double, C.c_double, C.c_int, C.POINTER(SolverOpts), C.POINTER(SolveStats)],
                       C.c_int),
    "ae_bottom_solve_noalloc": ([C.POINTER(LevelDesc), C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_void_p,
                                 C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int), C.c_void_p],
                                C.c_int),
    "ae_kernel_launches": ([], C.c_longlong),
    "ae_profile_kernel": ([P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "ae_batch_plan_bytes": ([C.POINTER(CellDesc), C.c_int], C.c_longlong),
    "ae_batch_create": ([C.POINTER(CellDesc), C.c_int, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "ae_batch_destroy": ([P], C.c_int),
    "ae_batch_num_solves": ([P], C.c_int),
    "ae_batch_num_levels": ([P, C.c_int], C.c_int),
    "ae_batch_device_bytes": ([P], C.c_longlong),
    "ae_batch_set_model": ([P, C.c_int, FAB], C.c_int),
    "ae_batch_set_model_grains": ([P, C.c_int, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "ae_batch_set_load": ([P, C.c_int, DP], C.c_int),
    "ae_batch_prepare": ([P], C.c_int),
    "ae_batch_solve": ([P, C.c_double, C.c_double, C.POINTER(SolverOpts), C.POINTER(CellStats)], C.c_int),
    "ae_batch_solution": ([P, C.c_int, FAB], C.c_int),
    "ae_batch_set_shape": ([P, C.c_int, C.c_int, C.c_int], C.c_int),
    "ae_batch_get_shape": ([P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "ae_server_default_opts": ([C.POINTER(ServerOpts)], None),
    "ae_server_create": ([C.c_int, C.POINTER(ServerOpts), C.POINTER(C.c_void_p)], C.c_int),
    "ae_server_destroy": ([P], C.c_int),
    "ae_server_submit": ([P, C.POINTER(CellDesc), C.c_int, C.c_void_p, C.c_void_p, FAB, DP,
                          C.POINTER(C.c_longlong)], C.c_int),
    "ae_server_poll": ([P, C.c_longlong, C.POINTER(RequestInfo), C.POINTER(CellStats), DP], C.c_int),
    "ae_server_wait": ([P, C.c_longlong, C.c_double, C.POINTER(RequestInfo), C.POINTER(CellStats), DP], C.c_int),
    "ae_server_release": ([P, C.c_longlong], C.c_int),
    "ae_server_get_stats": ([P, C.POINTER(ServerStats)], C.c_int),
    "ae_write_plotfile": ([C.c_char_p, C.c_int, C.POINTER(LevelDesc), FAB, C.c_int, C.POINTER(C.c_char_p),
                           C.c_double, C.POINTER(C.c_int)], C.c_int),
}

_lib = None


def load(path=None):
    """Load libaefast.so once; raise if it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libaefast.so not built at %s: run anisotropicfracture_gb300.build.build()" % path)
    lib = C.CDLL(path)
    for name, (argt, rest) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argt
        fn.restype = rest
    _lib = lib
    return lib


def check(code):
    if code != AE_OK:
        raise AeError(code, load().ae_last_error().decode())
    return code


def default_opts(**kw):
    o = SolverOpts()
    load().ae_default_solver_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o
