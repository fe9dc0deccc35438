"""Shared builders for the tests: seeded stiffness fields, BC tables and analytic fields."""
import numpy as np

from anisotropicfracture_gb300 import models
from anisotropicfracture_gb300.elastic import FACE, FACES, BCElastic

D, T, P, N = 0, 1, 2, 3


def random_coeffs(model, shape, rng, smooth=False):
    """Positive-definite-ish per-node stiffness of the given kind over `shape` (nz, ny, nx)."""
    if model == models.ISOTROPIC:
        lam = 1.0 + rng.random(shape)
        mu = 0.5 + rng.random(shape)
        return np.ascontiguousarray(np.stack([lam, mu]))
    if model == models.DIAGONAL:
        return np.ascontiguousarray(0.5 + rng.random((9,) + shape))
    Rs = models.random_rotations(4, rng)
    tabs = models.cubic(1.68, 1.21, 0.75, Rs)  # (4, 21)
    gid = rng.integers(0, 4, size=shape)
    C = np.moveaxis(tabs[gid], -1, 0)
    C = C * (0.8 + 0.4 * rng.random(shape))[None]
    return np.ascontiguousarray(C)


def bc_pull_z():
    """Pull along z: u = 0 on z = 0, u = (0, 0, 0.01) on z = 1, traction-free lateral faces;
    edges and corners touching z = 0 / z = 1 take the z-face type."""
    bc = BCElastic()
    for f in FACES:
        for d in range(3):
            bc.Set(f, d, D, 0.0)
    for f in ["XLO", "XHI", "YLO", "YHI", "XLO_YLO", "XLO_YHI", "XHI_YLO", "XHI_YHI"]:
        for d in range(3):
            bc.Set(f, d, T, 0.0)
    for f in FACES:
        if "ZHI" in f:
            bc.Set(f, 2, D, 0.01)
    return bc


def bc_random(rng):
    """Every face/edge/corner and direction gets a random type among displacement,
    traction and Neumann, and a random value."""
    bc = BCElastic()
    bc.type[:] = rng.choice([D, T, N], size=(26, 3))
    bc.val[:] = rng.standard_normal((26, 3))
    return bc


def bc_uniaxial_x():
    """BCs of src/Test/Operator/Elastic_UniaxialTest.cpp:205-238 (component 0, 3D)."""
    bc = BCElastic()
    X, Y, Z = 0, 1, 2
    bc.Set("XHI", X, D, 0.1); bc.Set("XHI", Y, N, 0.0); bc.Set("YLO", X, N, 0.0); bc.Set("YHI", X, N, 0.0)
    bc.Set("XHI_YHI", X, D, 0.1); bc.Set("XHI_YLO", X, D, 0.1)
    bc.Set("XHI", Z, N, 0.0); bc.Set("ZLO", X, N, 0.0); bc.Set("ZHI", X, N, 0.0)
    bc.Set("ZHI_XHI", X, D, 0.1); bc.Set("ZLO_XHI", X, D, 0.1)
    for c in ["XHI_YLO_ZLO", "XHI_YLO_ZHI", "XHI_YHI_ZLO", "XHI_YHI_ZHI"]:
        bc.Set(c, X, D, 0.1)
    for e in ["YLO_ZLO", "YLO_ZHI", "YHI_ZLO", "YHI_ZHI"]:
        bc.Set(e, X, N, 0.0)
        bc.Set(e, Y, N, 0.0)
    return bc


def node_coords(n, shape=None, dx=None):
    nz, ny, nx = shape if shape is not None else (n + 1,) * 3
    dx = 1.0 / n if dx is None else dx
    z, y, x = np.meshgrid(np.arange(nz) * dx, np.arange(ny) * dx, np.arange(nx) * dx, indexing="ij")
    return x, y, z


def normwise_err(a, ref):
    """max |a - ref| / max |ref|: the per-node error measured against the field's scale."""
    s = np.abs(ref).max()
    return float(np.abs(a - ref).max() / (s if s > 0 else 1.0))


def polycrystal_amr(n=16, nlev=2, seed=1):
    """The reference's test hierarchy (oracle amr_levels) with an 8-grain cubic Voronoi stiffness
    on every level (ghost nodes included) and the pull-along-z boundary values as right-hand sides."""
    from anisotropicfracture_gb300 import microstructure
    from oracle import pyoracle as po
    Ls = po.amr_levels(n, nlev)
    bc = bc_pull_z()
    seeds = microstructure.voronoi_seeds(8, seed)
    rot = models.random_rotations(8, np.random.default_rng(seed + 1))
    tab = models.cubic(1.68, 1.21, 0.75, rot)
    Cs, bs = [], []
    for L in Ls:
        lo = [L.lo[d] - L.ng for d in range(3)]
        hi = [L.hi[d] + L.ng for d in range(3)]
        gid = microstructure.voronoi_grain_ids(lo, hi, tuple(L.dx), seeds)
        Cs.append(np.ascontiguousarray(np.moveaxis(tab[gid], -1, 0)))
        bs.append(po.bc_init(L, bc.type, bc.val, np.zeros((3,) + L.shape)))
    return Ls, Cs, bc, bs


def golden_stiffness(parts):
    """The per-node stiffness of a golden case: stored whole, or as table[gid] * scale."""
    if "C" in parts:
        return np.ascontiguousarray(parts["C"])
    C = np.moveaxis(parts["tabs"][parts["gid"].astype(np.intp)], -1, 0) * parts["scale"][None]
    return np.ascontiguousarray(C)


def golden_case(z, name):
    """Case `name` ("iso", "mm", "diag" or "solve") of tests/golden/elastic_ops.npz as a dict
    with the keys the generator wrote, minus the prefix, plus the rebuilt stiffness "C"."""
    p = name + "_"
    d = {k[len(p):]: z[k] for k in z.files if k.startswith(p)}
    d["C"] = golden_stiffness(d)
    return d


# Per-node tolerance.  A node's error is measured against its own oracle value; nodes whose value
# is below PERNODE_FLOOR x max|oracle| (values produced by cancellation of much larger stencil
# terms, where a fused multiply-add on the GPU and a separate multiply and add in the oracle
# round differently) are measured against that floor instead.
PERNODE_FLOOR = 1e-3


def pernode_err(a, ref, floor=PERNODE_FLOOR):
    """max over nodes of |a - ref| / max(|ref_node|, floor * max|ref|)."""
    s = float(np.abs(ref).max())
    den = np.maximum(np.abs(ref), floor * (s if s > 0 else 1.0))
    return float((np.abs(a - ref) / den).max())


def pernode_report(a, ref):
    """The worst per-node relative error at the floors 0, 1e-9, 1e-6, 1e-3 (x max|oracle|)."""
    return {f: pernode_err(a, ref, f) for f in (0.0, 1e-9, 1e-6, 1e-3)}


def golden_level(z, lname):
    """The oracle level description stored as <lname>_level / <lname>_dxs in a fixture file."""
    from oracle import pyoracle as po
    v = [int(a) for a in z[lname + "_level"]]
    L = po.Level()
    for d in range(3):
        L.dom_lo[d], L.dom_hi[d], L.lo[d], L.hi[d] = v[d], v[3 + d], v[6 + d], v[9 + d]
        L.dx[d] = float(z[lname + "_dxs"][d])
    L.ng = v[12]
    return L


def golden_prefixed(z, prefix):
    """Entries of a fixture file whose key starts with `prefix`, without it, plus the rebuilt
    per-node stiffness "C" when the entries describe one."""
    d = {k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)}
    if "C" in d or "tabs" in d:
        d["C"] = golden_stiffness(d)
    return d
