"""Seeded synthetic microstructures for the benchmark configurations.

The reference's integrators build their per-node stiffness from initial-condition
classes; these generators follow the same semantics on nodal coordinates x = i * dx:
  sphere inclusion   IC::Sphere  (src/IC/Sphere.H:40-115): inside where |x - c|^2 < r^2
  Voronoi grains     IC::Voronoi (src/IC/Voronoi.H:47-101): nearest seed, Euclidean distance
All randomness comes from numpy Generators with the stated seeds.
"""
import numpy as np

from . import models


def node_grid(lo, hi, dx):
    """Nodal coordinates (z, y, x arrays, shape (nz, ny, nx)) of the index box [lo, hi]."""
    ax = [np.arange(lo[d], hi[d] + 1) * dx[d] for d in range(3)]
    return np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")


def sphere_indicator(lo, hi, dx, center=(0.5, 0.5, 0.5), radius=0.25, eps=None):
    """Inclusion order parameter eta in [0, 1].  eps = None: sharp node-in-sphere test
    (IC::Sphere, src/IC/Sphere.H:72-104).  eps > 0: the diffuse profile of IC::Ellipse,
    eta = 1/2 - 1/2 erf((x^T A x - 1) / (eps |A x|)) with A = I / r^2 (src/IC/Ellipse.H:70-71)."""
    Z, Y, X = node_grid(lo, hi, dx)
    rsq = (X - center[0]) ** 2 + (Y - center[1]) ** 2 + (Z - center[2]) ** 2
    if eps is None:
        return (rsq < radius * radius).astype(np.float64)
    from scipy.special import erf
    q = (rsq - radius * radius) / (radius * radius)
    nrm = np.maximum(np.sqrt(rsq) / (radius * radius), 1e-300)
    return 0.5 - 0.5 * erf(q / eps / nrm)


def sphere_inclusion_iso(lo, hi, dx, center=(0.5, 0.5, 0.5), radius=0.25, E_in=10.0, nu_in=0.3, E_out=1.0,
                         nu_out=0.3, eps_cells=2.0):
    """(lambda, mu) per node, shape (2, nz, ny, nx): (1 - eta) matrix + eta inclusion, the
    mixture the Eshelby integrator forms from its eta field (src/Integrator/Eshelby.H:108-118).
    eps_cells = interface width in cells (None: sharp).  A sharp 10:1 jump makes the
    reference's damped-Jacobi smoother diverge (the non-divergence-form grad C term), so the
    configurations use a 2-cell diffuse interface."""
    eps = None if eps_cells is None else eps_cells * dx[0]
    eta = sphere_indicator(lo, hi, dx, center, radius, eps)
    li, mi = models.lame_from_E_nu(E_in, nu_in)
    lo_, mo = models.lame_from_E_nu(E_out, nu_out)
    out = np.empty((2,) + eta.shape)
    out[0] = (1.0 - eta) * lo_ + eta * li
    out[1] = (1.0 - eta) * mo + eta * mi
    return out


def voronoi_seeds(nseeds, seed, extent=(1.0, 1.0, 1.0)):
    rng = np.random.default_rng(seed)
    return rng.random((nseeds, 3)) * np.asarray(extent)[None, :]


def voronoi_grain_ids(lo, hi, dx, seeds, periodic_extent=None, chunk=1 << 20):
    """Grain id (nearest seed) of every node of the box [lo, hi]; int32 (nz, ny, nx).
    periodic_extent: box size for a periodic (minimum-image) distance, or None."""
    try:
        from scipy.spatial import cKDTree
    except ImportError:  # pragma: no cover
        cKDTree = None
    Z, Y, X = node_grid(lo, hi, dx)
    pts = np.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], axis=1)
    if periodic_extent is not None:
        ext = np.asarray(periodic_extent, dtype=np.float64)
        pts = np.mod(pts, ext)
    out = np.empty(pts.shape[0], dtype=np.int32)
    if cKDTree is not None:
        tree = cKDTree(seeds, boxsize=None if periodic_extent is None else np.asarray(periodic_extent) + 0.0)
        for s in range(0, pts.shape[0], chunk):
            out[s:s + chunk] = tree.query(pts[s:s + chunk], k=1)[1]
    else:
        for s in range(0, pts.shape[0], chunk):
            p = pts[s:s + chunk]
            d = ((p[:, None, :] - seeds[None, :, :]) ** 2).sum(-1)
            out[s:s + chunk] = np.argmin(d, axis=1)
    return out.reshape(Z.shape)


def cubic_polycrystal(lo, hi, dx, nseeds=64, seed_points=1, seed_rot=2, C11=1.68, C12=1.21, C44=0.75,
                      extent=(1.0, 1.0, 1.0), periodic=False):
    """21-slot cubic stiffness per node over [lo, hi]: Voronoi grains (seed_points) with
    Haar-uniform rotations (seed_rot).  Returns (C (21, nz, ny, nx), grain ids, table (G, 21))."""
    seeds = voronoi_seeds(nseeds, seed_points, extent)
    gid = voronoi_grain_ids(lo, hi, dx, seeds, periodic_extent=extent if periodic else None)
    rot = models.random_rotations(nseeds, np.random.default_rng(seed_rot))
    table = models.cubic(C11, C12, C44, rot)
    C = np.ascontiguousarray(np.moveaxis(table[gid], -1, 0))
    return C, gid, table


def penny_crack_damage(lo, hi, dx, ncracks=8, seed=3, rmin=0.1, rmax=0.2, width_cells=3.0, cell=None):
    """Damage c in [0, 1]: clamped sum over cracks of exp(-(d_n / l)^2) inside each disc,
    d_n the distance to the crack plane, l = width_cells * cell size."""
    rng = np.random.default_rng(seed)
    cell = dx[0] if cell is None else cell
    ell = width_cells * cell
    Z, Y, X = node_grid(lo, hi, dx)
    c = np.zeros(X.shape)
    centers = rng.random((ncracks, 3))
    normals = rng.standard_normal((ncracks, 3))
    normals /= np.linalg.norm(normals, axis=1)[:, None]
    radii = rmin + (rmax - rmin) * rng.random(ncracks)
    for q in range(ncracks):
        dxv, dyv, dzv = X - centers[q, 0], Y - centers[q, 1], Z - centers[q, 2]
        dn = dxv * normals[q, 0] + dyv * normals[q, 1] + dzv * normals[q, 2]
        inplane2 = dxv * dxv + dyv * dyv + dzv * dzv - dn * dn
        c += np.where(inplane2 <= radii[q] ** 2, np.exp(-(dn / ell) ** 2), 0.0)
    return np.clip(c, 0.0, 1.0)
