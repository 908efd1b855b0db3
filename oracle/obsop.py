"""Restatement of the along-track observation operator of the reference
(mapping/src/obsop.py, Obsop_interp_l3_jax, and the neighbour rules of the
scipy Obsop_interp_l3) in float64 NumPy. Test
infrastructure only.

Planar coordinates: the reference maps lon/lat to 3-D Cartesian km
(grid.geo2cart, obsop.py:421-422) before its KDTree query; the synthetic
Cartesian grids here use planar x/y in km directly, with the same
Npix-nearest search, distance cut ``dmax`` (obsop.py:406) and Gaussian weights
(obsop.py:433-445). The ``*_points`` forms take any Cartesian coordinates,
and ``geo2cart`` restates grid.py:61-98. Parity: the neighbours, weights,
dmax, exclusions and ``geo2cart`` are pinned to golden vectors produced by the
reference's own obsop.py and grid.py on a lon/lat grid
(tests/golden/gen_golden_obs.py); the misfit and its adjoint are checked by
transposition and finite differences.
"""
import numpy as np
from scipy.spatial import cKDTree


def dmax_km(dx, dy, npix):
    """Maximal interpolation distance of obsop.py:406 for uniform spacing [m]."""
    return npix * np.sqrt(dx ** 2 + dy ** 2) * 1e-3 * np.sqrt(2) / 2


def dmax_from_metrics(DX, DY, npix):
    """obsop.py:406 (and 194) for grid spacing arrays DX, DY [m]."""
    return npix * np.mean(np.sqrt(np.asarray(DX) ** 2 + np.asarray(DY) ** 2)) * 1e-3 * np.sqrt(2) / 2


def geo2cart(lonlat):
    """Geodetic (lon, lat) in degrees to Cartesian km on the WGS 84 ellipsoid
    at zero height (grid.py:61-98)."""
    c = np.atleast_2d(np.asarray(lonlat, dtype=np.float64))
    lat, lon = np.radians(c[:, 1]), np.radians(c[:, 0])
    a, e2 = 6378.137, 6.69437999014e-3
    rn = a / np.sqrt(1 - e2 * np.sin(lat) ** 2)
    return np.column_stack((rn * np.cos(lat) * np.cos(lon), rn * np.cos(lat) * np.sin(lon),
                            rn * (1 - e2) * np.sin(lat)))


def _planar(ny, nx, dx, dy):
    gx, gy = np.meshgrid(np.arange(nx) * dx / 1e3, np.arange(ny) * dy / 1e3)
    return np.column_stack((gx.ravel(), gy.ravel()))


def sparse_op(x_obs_km, y_obs_km, ny, nx, dx, dy, npix=4):
    """(data, rows, cols) of H following obsop.py:417-460 on the planar grid."""
    return sparse_op_points(_planar(ny, nx, dx, dy), np.column_stack((x_obs_km, y_obs_km)), npix,
                            dmax_km(dx, dy, npix))


def sparse_op_points(grid_pts, obs_pts, npix, dmax):
    """(data, rows, cols) of the jax operator's H (obsop.py:417-460) for grid
    and observation points in any Cartesian coordinates (km): the ``npix``
    nearest grid points, those within ``dmax`` kept, Gaussian weights
    normalised per observation (npix = 1: weight 1). Entries are ordered by
    observation, then by distance.

    For npix = 1 the reference returns an empty operator: its KDTree query
    then gives 1-D arrays, ``row, col = np.where(valid_mask)`` cannot unpack
    one index array, and the bare ``except`` (obsop.py:452-458) yields no
    entries. This restatement keeps the nearest point with weight 1, the
    evident intent, as the library does."""
    tree = cKDTree(np.asarray(grid_pts, dtype=np.float64))
    D, ind = tree.query(np.asarray(obs_pts, dtype=np.float64), k=npix)
    if npix == 1:
        D, ind = D[:, None], ind[:, None]
    valid = D <= dmax
    if npix > 1:
        w = np.exp(-D ** 2 / (2 * (0.5 * dmax) ** 2)) * valid
        s = np.sum(w, axis=1, keepdims=True)
        w = np.divide(w, s, out=np.zeros_like(w), where=s > 0)
    else:
        w = np.ones_like(D)
    rows, cols = np.where(valid)
    return w[rows, cols], rows, ind[rows, cols]


def misfit(x_flat, data, rows, cols, yobs, err):
    """inverr*(Hx - y) with NaN -> 0 (obsop.py:610-628)."""
    hx = np.zeros(yobs.size)
    np.add.at(hx, rows, data * x_flat[cols])
    m = hx - yobs
    inverr = 1.0 / err
    m = np.where(np.isnan(m), 0, m)
    inverr = np.where(np.isnan(inverr), 0, inverr)
    return inverr * m


def misfit_adj(cot, data, rows, cols, err, size, x_flat=None, yobs=None):
    """vjp of :func:`misfit` w.r.t. x at cotangent ``cot`` (obsop.py:630-678).
    Entries whose misfit was NaN pass no derivative."""
    inverr = np.where(np.isnan(1.0 / err), 0, 1.0 / err)
    g = inverr * cot
    if x_flat is not None:
        hx = np.zeros(cot.size)
        np.add.at(hx, rows, data * x_flat[cols])
        g = np.where(np.isnan(hx - yobs), 0, g)
    ad = np.zeros(size)
    np.add.at(ad, cols, data * g[rows])
    return ad


def l3_excluded_coords(X, Y, mask=None, mask_borders=False):
    """:func:`l3_excluded` for grid coordinates X, Y [ny, nx] of any kind
    (lon/lat in the reference, obsop.py:118-134)."""
    out = set()
    if mask is not None:
        out.update(int(j) for j in np.where(np.asarray(mask))[1])
    if mask_borders:
        ring = np.column_stack((np.concatenate((X[0, :], X[1:-1, -1], X[-1, :], X[:, 0])),
                                np.concatenate((Y[0, :], Y[1:-1, -1], Y[-1, :], Y[:, 0]))))
        pts = np.column_stack((X.ravel(), Y.ravel()))
        for i in range(pts.shape[0]):
            if np.any(np.all(np.isclose(ring, pts[i]), axis=1)):
                out.add(i)
    return out


def l3_excluded(ny, nx, dx, dy, mask=None, mask_borders=False):
    """Flat grid indices the scipy operator ``Obsop_interp_l3`` skips when it
    picks neighbours (obsop.py:118-134), on the planar grid of this module.

    ``ind_mask`` is ``np.where(State.mask)[1]`` (obsop.py:120): for a 2-D mask
    that is the COLUMN number of every masked point, compared later with flat
    indices, so the points it removes are those of row 0 whose column holds a
    masked point. ``ind_borders`` is every point whose coordinates are close
    (np.isclose) to those of a point on the outer ring (obsop.py:126-134)."""
    gx, gy = np.meshgrid(np.arange(nx) * dx / 1e3, np.arange(ny) * dy / 1e3)
    return l3_excluded_coords(gx, gy, mask, mask_borders)


def sparse_op_l3(x_obs_km, y_obs_km, ny, nx, dx, dy, npix=4, excluded=()):
    """(data, rows, cols) of the scipy operator's H (``_sparse_op``,
    obsop.py:197-219): per observation, all grid distances, the ``npix``
    nearest in order; a neighbour is kept if it is not excluded and lies
    within ``dmax``; kept weights exp(-d^2/(2(dmax/2)^2)) normalised over the
    kept ones. Excluded neighbours keep their place among the ``npix``
    nearest (they are not replaced by the next one). Equal distances are
    ordered by grid index (the reference's argsort leaves them unordered;
    they do not occur at seeded random positions)."""
    return sparse_op_l3_points(_planar(ny, nx, dx, dy), np.column_stack((x_obs_km, y_obs_km)), npix,
                               dmax_km(dx, dy, npix), excluded)


def sparse_op_l3_points(grid_pts, obs_pts, npix, dmax, excluded=()):
    """:func:`sparse_op_l3` for grid and observation points in any Cartesian
    coordinates (km; the reference uses grid.geo2cart of lon/lat)."""
    grid = np.asarray(grid_pts, dtype=np.float64)
    obs = np.asarray(obs_pts, dtype=np.float64)
    excluded = set(excluded)
    data, rows, cols = [], [], []
    for o in range(obs.shape[0]):
        dist = np.sqrt(((grid - obs[o]) ** 2).sum(axis=1))
        order = np.argsort(dist, kind="stable")
        ws = []
        for p in range(npix):
            k = int(order[p])
            if k not in excluded and dist[k] <= dmax:
                ws.append(np.exp(-(dist[k] ** 2 / (2 * (0.5 * dmax) ** 2))))
                rows.append(o)
                cols.append(k)
        s = np.sum(ws)
        data.extend(w / s for w in ws)
    return np.asarray(data, dtype=np.float64), np.asarray(rows, dtype=np.int64), np.asarray(cols, dtype=np.int64)
