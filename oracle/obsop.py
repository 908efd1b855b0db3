"""Restatement of the along-track observation operator of the reference
(mapping/src/obsop.py, Obsop_interp_l3_jax) in float64 NumPy. Test
infrastructure only.

Planar coordinates: the reference maps lon/lat to 3-D Cartesian km
(grid.geo2cart, obsop.py:421-422) before its KDTree query; the synthetic
Cartesian grids here use planar x/y in km directly, with the same
Npix-nearest search, distance cut ``dmax`` (obsop.py:406) and Gaussian weights
(obsop.py:433-445). Parity: unpinned (the reference ships no golden values for
this operator and jax is not importable); checked by transposition and
finite-difference tests.
"""
import numpy as np
from scipy.spatial import cKDTree


def dmax_km(dx, dy, npix):
    """Maximal interpolation distance of obsop.py:406 for uniform spacing [m]."""
    return npix * np.sqrt(dx ** 2 + dy ** 2) * 1e-3 * np.sqrt(2) / 2


def sparse_op(x_obs_km, y_obs_km, ny, nx, dx, dy, npix=4):
    """(data, rows, cols) of H following obsop.py:417-460."""
    gx, gy = np.meshgrid(np.arange(nx) * dx / 1e3, np.arange(ny) * dy / 1e3)
    tree = cKDTree(np.column_stack((gx.ravel(), gy.ravel())))
    D, ind = tree.query(np.column_stack((x_obs_km, y_obs_km)), k=npix)
    if npix == 1:
        D, ind = D[:, None], ind[:, None]
    dmax = dmax_km(dx, dy, npix)
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
