"""Batched periodic cells (RVE homogenisation) over the C ABI's ae_batch_* entry points.

A cell is a periodic box of n[0] x n[1] x n[2] nodes (x = i * length / n); each solve on a cell
imposes a macroscopic displacement gradient E (3x3) and finds the periodic fluctuation w with
A w + c = b, mean(w) = 0 (c: a uniform body force), b = -sum_d (d_d C) : E e_d, the interior row of
Operator::Elastic<T>::Fapply (src/Operator/Elastic.cpp:216-255) at every node with periodic
neighbours.  All solves of a batch advance together on the device.

Fields are numpy arrays (host) or torch CUDA tensors shaped (ncomp, nz, ny, nx), i fastest.
"""
import ctypes as C

import numpy as np

from . import _lib, models
from .elastic import Field


def cell_desc(n, nrhs=1, length=1.0):
    d = _lib.CellDesc()
    n = (n,) * 3 if np.isscalar(n) else tuple(n)
    length = (length,) * 3 if np.isscalar(length) else tuple(length)
    for k in range(3):
        d.n[k] = int(n[k])
        d.length[k] = float(length[k])
    d.nrhs = int(nrhs)
    return d


def plan_bytes(n, nrhs=1, model=models.MAJORMINOR):
    """Device bytes one cell needs (its hierarchy and nrhs solves)."""
    d = cell_desc(n, nrhs)
    return int(_lib.load().ae_batch_plan_bytes(C.byref(d), model))


def stats_dict(s):
    return {"iters": s.iters, "converged": bool(s.converged), "nlevels": s.nlevels, "bottom_fail": s.bottom_fail,
            "res0": s.res0, "resfinal": s.resfinal, "target": s.target, "seconds": s.seconds,
            "body_force": np.array(s.body_force[:]), "mean_stress": np.array(s.mean_stress[:]).reshape(3, 3)}


class CellBatch:
    """A set of periodic cells and their load cases, solved together (ae_batch_*)."""

    def __init__(self, cells, model=models.MAJORMINOR):
        """cells: list of (n, nrhs) or (n, nrhs, length); n an int or 3 ints."""
        self.lib = _lib.load()
        self.model = model
        self.ncoef = models.NCOEF[model]
        descs = [cell_desc(*c) if isinstance(c, (tuple, list)) else cell_desc(c) for c in cells]
        arr = (_lib.CellDesc * len(descs))(*descs)
        h = C.c_void_p()
        _lib.check(self.lib.ae_batch_create(arr, len(descs), model, C.byref(h)))
        self.handle = h
        self.descs = descs
        self.nsolves = self.lib.ae_batch_num_solves(h)
        self.solve_cell = []
        for c, d in enumerate(descs):
            self.solve_cell += [c] * d.nrhs

    def shape_of(self, cell):
        d = self.descs[cell]
        return (d.n[2], d.n[1], d.n[0])

    def num_levels(self, cell):
        return self.lib.ae_batch_num_levels(self.handle, cell)

    def device_bytes(self):
        return int(self.lib.ae_batch_device_bytes(self.handle))

    def set_model(self, cell, Cf):
        f = Field(Cf).fab()
        _lib.check(self.lib.ae_batch_set_model(self.handle, cell, C.byref(f)))

    def set_grains(self, cell, seeds, table):
        seeds = np.ascontiguousarray(seeds, dtype=np.float64)
        table = np.ascontiguousarray(table, dtype=np.float64)
        assert seeds.shape[1] == 3 and table.shape == (seeds.shape[0], self.ncoef)
        _lib.check(self.lib.ae_batch_set_model_grains(self.handle, cell, seeds.shape[0], seeds.ctypes.data,
                                                      table.ctypes.data))

    def set_load(self, solve, E):
        E = np.ascontiguousarray(E, dtype=np.float64).reshape(9)
        _lib.check(self.lib.ae_batch_set_load(self.handle, solve, E.ctypes.data_as(C.POINTER(C.c_double))))

    def prepare(self):
        _lib.check(self.lib.ae_batch_prepare(self.handle))

    def solve(self, tol_rel=1e-8, tol_abs=0.0, check=True, **opts):
        """Solve every load case; returns (list of per-solve stats dicts, status code)."""
        o = _lib.default_opts(**opts)
        st = (_lib.CellStats * self.nsolves)()
        rc = self.lib.ae_batch_solve(self.handle, tol_rel, tol_abs, C.byref(o), st)
        if check and rc != _lib.AE_OK:
            _lib.check(rc)
        return [stats_dict(s) for s in st], rc

    def solution(self, solve, out=None):
        c = self.solve_cell[solve]
        if out is None:
            out = np.zeros((3,) + self.shape_of(c))
        f = Field(out).fab()
        _lib.check(self.lib.ae_batch_solution(self.handle, solve, C.byref(f)))
        return out

    def set_shape(self, level, chunk, grid):
        _lib.check(self.lib.ae_batch_set_shape(self.handle, level, chunk, grid))

    def get_shape(self, level):
        c, g = C.c_int(), C.c_int()
        _lib.check(self.lib.ae_batch_get_shape(self.handle, level, C.byref(c), C.byref(g)))
        return c.value, g.value

    def close(self):
        if self.handle:
            self.lib.ae_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CellServer:
    """Continuous-batching request loop for cell homogenisation (ae_server_*)."""

    QUEUED, RUNNING = 1, 2

    def __init__(self, model=models.MAJORMINOR, hbm_budget_bytes=0, max_live_solves=0, keep_solution=False,
                 tol_rel=1e-8, tol_abs=0.0, **solver):
        self.lib = _lib.load()
        self.model = model
        self.ncoef = models.NCOEF[model]
        o = _lib.ServerOpts()
        self.lib.ae_server_default_opts(C.byref(o))
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        o.max_live_solves = int(max_live_solves)
        o.keep_solution = int(bool(keep_solution))
        o.tol_rel, o.tol_abs = tol_rel, tol_abs
        for k, v in solver.items():
            if not hasattr(o.solver, k):
                raise KeyError(k)
            setattr(o.solver, k, v)
        h = C.c_void_p()
        _lib.check(self.lib.ae_server_create(model, C.byref(o), C.byref(h)))
        self.handle = h
        self.keep_solution = bool(keep_solution)
        self._shape = {}

    def submit(self, n, loads, seeds=None, table=None, field=None, length=1.0):
        """Queue one cell; loads: list of 3x3 gradients.  Returns the ticket."""
        d = cell_desc(n, len(loads), length)
        E = np.ascontiguousarray(np.stack([np.asarray(e, dtype=np.float64).reshape(9) for e in loads]))
        t = C.c_longlong()
        if field is None:
            seeds = np.ascontiguousarray(seeds, dtype=np.float64)
            table = np.ascontiguousarray(table, dtype=np.float64)
            rc = self.lib.ae_server_submit(self.handle, C.byref(d), seeds.shape[0], seeds.ctypes.data,
                                           table.ctypes.data, None, E.ctypes.data_as(C.POINTER(C.c_double)),
                                           C.byref(t))
        else:
            f = Field(np.ascontiguousarray(field, dtype=np.float64)).fab()
            rc = self.lib.ae_server_submit(self.handle, C.byref(d), 0, None, None, C.byref(f),
                                           E.ctypes.data_as(C.POINTER(C.c_double)), C.byref(t))
        _lib.check(rc)
        self._shape[t.value] = (len(loads), (d.n[2], d.n[1], d.n[0]))
        return t.value

    def _result(self, ticket, info, st, w):
        out = {"status": info.status, "t_submit": info.t_submit, "t_admit": info.t_admit, "t_done": info.t_done,
               "latency": info.latency}
        if info.status <= 0:
            out["stats"] = [stats_dict(s) for s in st]
            if w is not None:
                nrhs, shp = self._shape[ticket]
                out["w"] = w.reshape((nrhs, 3) + shp)
        return out

    def _buffers(self, ticket):
        if ticket not in self._shape:  # unknown or released: the library reports the error
            return (_lib.CellStats * 1)(), None
        nrhs, shp = self._shape[ticket]
        st = (_lib.CellStats * nrhs)()
        w = np.zeros(nrhs * 3 * int(np.prod(shp))) if self.keep_solution else None
        return st, w

    def poll(self, ticket):
        info = _lib.RequestInfo()
        st, w = self._buffers(ticket)
        _lib.check(self.lib.ae_server_poll(self.handle, ticket, C.byref(info), st,
                                           None if w is None else w.ctypes.data_as(C.POINTER(C.c_double))))
        return self._result(ticket, info, st, w)

    def wait(self, ticket, timeout=-1.0):
        info = _lib.RequestInfo()
        st, w = self._buffers(ticket)
        _lib.check(self.lib.ae_server_wait(self.handle, ticket, float(timeout), C.byref(info), st,
                                           None if w is None else w.ctypes.data_as(C.POINTER(C.c_double))))
        return self._result(ticket, info, st, w)

    def release(self, ticket):
        _lib.check(self.lib.ae_server_release(self.handle, ticket))
        self._shape.pop(ticket, None)

    def stats(self):
        s = _lib.ServerStats()
        _lib.check(self.lib.ae_server_get_stats(self.handle, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if self.handle:
            self.lib.ae_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- multi-GPU sharding
def partition_cells(cell_bytes, nranks):
    """Assign cells to ranks: largest first, each to the rank with the fewest bytes so far (ties
    to the lower rank).  Deterministic, so every rank computes the same assignment without a
    collective.  Returns one list of cell indices per rank, each in increasing order."""
    order = sorted(range(len(cell_bytes)), key=lambda c: (-cell_bytes[c], c))
    load = [0] * nranks
    parts = [[] for _ in range(nranks)]
    for c in order:
        r = min(range(nranks), key=lambda q: (load[q], q))
        parts[r].append(c)
        load[r] += cell_bytes[c]
    return [sorted(p) for p in parts]


# ---------------------------------------------------------------- synthetic cells
def rve_grains(n, ngrains, seed, length=1.0, C11=1.68, C12=1.21, C44=0.75):
    """Seeds (ngrains x 3, uniform in the cell) and cubic tables (Haar-uniform rotations) of a
    periodic polycrystal cell; seed drives both draws."""
    rng = np.random.default_rng(seed)
    seeds = rng.random((ngrains, 3)) * length
    table = models.cubic(C11, C12, C44, models.random_rotations(ngrains, rng))
    return seeds, table


def rve_stiffness(n, seeds, table, length=1.0):
    """Host-side per-node stiffness of a periodic Voronoi cell (nearest seed, minimum image),
    shape (ncoef, n, n, n): the same map the device builds in ae_batch_set_model_grains."""
    from .microstructure import voronoi_grain_ids
    dx = (length / n,) * 3
    gid = voronoi_grain_ids((0, 0, 0), (n - 1,) * 3, dx, seeds, periodic_extent=(length,) * 3)
    return np.ascontiguousarray(np.moveaxis(table[gid], -1, 0))


def unit_strains(eps=1e-3):
    """The six unit macroscopic strains (normal xx, yy, zz; shear yz, zx, xy) times eps, as 3x3
    symmetric displacement gradients."""
    out = []
    for a, b in [(0, 0), (1, 1), (2, 2), (1, 2), (2, 0), (0, 1)]:
        E = np.zeros((3, 3))
        E[a, b] += eps / (1.0 if a == b else 2.0)
        if a != b:
            E[b, a] += eps / 2.0
        out.append(E)
    return out
