"""ae_bottom_solve_noalloc: the bottom (coarsest-level) solve for callers that cannot allocate
device memory, e.g. an application whose memory arena already owns the GPU but runs its own
multigrid and needs our coarse-grid solve.  Its work space is a fixed array inside the library.

Checked through the C ABI against the existing entry point ae_solve on the same level: with odd
cell counts the level has one multigrid level, so ae_solve's first iteration is exactly one
bottom solve of the right-hand side (the solution starts from zero).  Two calls in a row with
different inputs, CG (which fails on this non-symmetric operator and falls back to smoothing)
and BiCGStab, cubic per-node stiffness and a uniform isotropic one (m_uniform).  Tolerance: the
FP64 parity bound of the other GPU tests, 1e-12 of the max-norm.  The device's free memory is the
same before and after the calls: the entry point allocates nothing."""
import ctypes as C

import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, models
from anisotropicfracture_gb300.elastic import BCElastic, Elastic, Field, level_desc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12
CELLS = (7, 7, 7)  # 512 nodes, one multigrid level


def _case(seed, model=models.MAJORMINOR):
    rng = np.random.default_rng(seed)
    shape = tuple(c + 1 for c in CELLS[::-1])
    if model == models.MAJORMINOR:
        tabs = models.cubic(1.68, 1.21, 0.75, models.random_rotations(3, rng))
        gid = rng.integers(0, 3, size=shape)
        Cf = np.ascontiguousarray(np.moveaxis(tabs[gid], -1, 0))
    else:  # one isotropic material everywhere
        Cf = np.empty((2,) + shape)
        Cf[0], Cf[1] = 1.0 + rng.random(), 0.5 + rng.random()
    b = rng.standard_normal((3,) + shape)
    bc = BCElastic()
    for f in ["XLO", "XHI", "YLO", "YHI", "XLO_YLO", "XLO_YHI", "XHI_YLO", "XHI_YHI"]:
        for d in range(3):
            bc.Set(f, d, bc.Traction, 0.0)
    return Cf, b, bc


def _existing_entry_point(Cf, b, bc, bottom, model=models.MAJORMINOR, uniform=False):
    op = Elastic([level_desc(CELLS)], model)
    op.SetModel(0, Field(Cf))
    op.SetBC(bc)
    op.SetUniform(uniform)
    assert op.NMGLevels(0) == 1
    opts = _lib.default_opts(max_fmg_iter=0, bottom=bottom, max_iter=1, bottom_max_iter=200, bottom_reltol=1e-4,
                             nuf=8, sweeps=2, use_graph=0)
    x = np.zeros_like(b)
    fs, fr = Field(x).fab(), Field(b).fab()
    st = _lib.SolveStats()
    rc = _lib.load().ae_solve(op.handle, C.byref(fs), C.byref(fr), 1e-30, 0.0, C.byref(opts), C.byref(st))
    assert rc in (_lib.AE_OK, _lib.AE_ERR_NOT_CONVERGED)
    op.close()
    return x, st.bottom_fail


def _call(Cd, bd, xd, bc, bottom, model, uniform):
    """One call of the entry point on device tensors; returns its Krylov failure count."""
    L = level_desc(CELLS)
    bt = np.ascontiguousarray(bc.type, dtype=np.int32)
    failed = C.c_int(-1)
    rc = _lib.load().ae_bottom_solve_noalloc(C.byref(L), model, C.c_void_p(Cd.data_ptr()),
                                             bt.ctypes.data_as(C.POINTER(C.c_int)), int(uniform),
                                             C.c_void_p(bd.data_ptr()), C.c_void_p(xd.data_ptr()), bottom, 200,
                                             1e-4, 8, C.byref(failed), None)
    _lib.check(rc)
    return failed.value


def _noalloc(Cf, b, bc, bottom, model=models.MAJORMINOR, uniform=False):
    Cd = torch.from_numpy(Cf).cuda()
    bd = torch.from_numpy(b).cuda()
    xd = torch.full_like(bd, 7.0)  # stale contents: the entry point must start from zero
    torch.cuda.synchronize()
    failed = _call(Cd, bd, xd, bc, bottom, model, uniform)
    return xd.cpu().numpy(), failed


@pytest.mark.parametrize("model,uniform", [(models.MAJORMINOR, False), (models.ISOTROPIC, True)])
@pytest.mark.parametrize("bottom", [0, 1])
def test_noalloc_bottom_solve_matches_existing_entry_point(bottom, model, uniform):
    for seed in (1, 2):  # two calls in a row share the one work space
        Cf, b, bc = _case(seed, model)
        ref, ref_fail = _existing_entry_point(Cf, b, bc, bottom, model, uniform)
        x, failed = _noalloc(Cf, b, bc, bottom, model, uniform)
        scale = np.abs(ref).max()
        assert scale > 0
        assert np.abs(x - ref).max() <= TOL64 * scale
        assert failed == ref_fail


def test_noalloc_leaves_device_memory_unchanged():
    """Inputs are placed first; across two calls the device's free memory must not move."""
    Cf, b, bc = _case(3)
    Cd = torch.from_numpy(Cf).cuda()
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros_like(bd)
    _call(Cd, bd, xd, bc, 1, models.MAJORMINOR, False)  # the first call on the device sets up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for bottom in (0, 1):
        _call(Cd, bd, xd, bc, bottom, models.MAJORMINOR, False)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_levels_beyond_its_work_space():
    lib = _lib.load()
    L = level_desc((17, 17, 17))  # 18^3 = 5832 nodes > AE_NOALLOC_MAX_NODES
    bt = np.zeros((26, 3), np.int32)
    rc = lib.ae_bottom_solve_noalloc(C.byref(L), models.MAJORMINOR, C.c_void_p(8), bt.ctypes.data_as(C.POINTER(C.c_int)),
                                     0, C.c_void_p(8), C.c_void_p(8), 0, 200, 1e-4, 8, None, None)
    assert rc == _lib.AE_ERR_ARG
    assert b"4913" in lib.ae_last_error()
    # sizes whose node count would overflow a 64-bit product are rejected the same way
    L = level_desc((1 << 30, 1 << 30, 1 << 30))
    rc = lib.ae_bottom_solve_noalloc(C.byref(L), models.MAJORMINOR, C.c_void_p(8), bt.ctypes.data_as(C.POINTER(C.c_int)),
                                     0, C.c_void_p(8), C.c_void_p(8), 0, 200, 1e-4, 8, None, None)
    assert rc == _lib.AE_ERR_ARG
