"""The observation-operator restatement (oracle/obsop.py) and the library's
exclusion table against golden vectors produced by the reference's own
obsop.py and grid.py (tests/golden/gen_golden_obs.py): both operator forms
on a lon/lat grid with land, with and without masked borders."""
import os

import numpy as np
import pytest

from oracle import obsop as ob
from vardyn_gb300.obsop import l3_exclusion

GOLD = os.path.join(os.path.dirname(__file__), "golden", "obs_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _case(g, t):
    lon, lat = np.meshgrid(g[f"{t}_lon"], g[f"{t}_lat"])
    obs = ob.geo2cart(np.column_stack((g[f"{t}_lon_obs"], g[f"{t}_lat_obs"])))
    grid = ob.geo2cart(np.column_stack((lon.ravel(), lat.ravel())))
    DX = np.radians(g[f"{t}_lon"][1] - g[f"{t}_lon"][0]) * 6371e3 * np.cos(np.radians(lat))
    DY = np.full(lon.shape, np.radians(g[f"{t}_lat"][1] - g[f"{t}_lat"][0]) * 6371e3)
    return lon, lat, grid, obs, DX, DY


def _sorted(data, rows, cols):
    o = np.lexsort((cols, rows))
    return np.asarray(data)[o], np.asarray(rows)[o], np.asarray(cols)[o]


def test_geo2cart_matches_reference(g):
    got = ob.geo2cart(g["geo2cart_in"])
    assert np.abs(got - g["geo2cart_out"]).max() <= 1e-12 * np.abs(g["geo2cart_out"]).max()


@pytest.mark.parametrize("t,borders", [("a", False), ("b", True)])
def test_excluded_points_match_reference(g, t, borders):
    lon, lat, *_ = _case(g, t)
    ref = set(g[f"{t}_ind_mask"].tolist()) | set(g[f"{t}_ind_borders"].tolist())
    assert ob.l3_excluded_coords(lon, lat, g[f"{t}_mask"], borders) == ref
    ny, nx = lon.shape
    assert set(np.flatnonzero(l3_exclusion(ny, nx, g[f"{t}_mask"], borders)).tolist()) == ref


@pytest.mark.parametrize("t,borders", [("a", False), ("b", True)])
@pytest.mark.parametrize("npix", [4, 1])
def test_scipy_operator_matches_reference(g, t, borders, npix):
    lon, lat, grid, obs, DX, DY = _case(g, t)
    dmax = ob.dmax_from_metrics(DX, DY, npix)
    assert abs(dmax - g[f"{t}_dmax_n{npix}"]) <= 1e-14 * dmax
    excl = ob.l3_excluded_coords(lon, lat, g[f"{t}_mask"], borders)
    d, r, c = _sorted(*ob.sparse_op_l3_points(grid, obs, npix, dmax, excl))
    p = f"{t}_l3_n{npix}_"
    assert np.array_equal(r, g[p + "row"]) and np.array_equal(c, g[p + "col"])
    assert np.abs(d - g[p + "data"]).max() <= 1e-15


@pytest.mark.parametrize("t", ["a", "b"])
def test_jax_operator_matches_reference(g, t):
    lon, lat, grid, obs, DX, DY = _case(g, t)
    d, r, c = ob.sparse_op_points(grid, obs, 4, ob.dmax_from_metrics(DX, DY, 4))
    ind = g[f"{t}_jax_n4_indices"]
    assert np.array_equal(r, ind[0]) and np.array_equal(c, ind[1])
    assert np.abs(d - g[f"{t}_jax_n4_data"]).max() <= 1e-15


def test_reference_jax_operator_is_empty_for_one_neighbour(g):
    """The reference's jax operator with npix = 1 has no entries (its
    np.where unpacking fails inside a bare except); the restatement keeps the
    nearest point with weight 1 instead."""
    assert g["a_jax_n1_data"].size == 0 and g["b_jax_n1_data"].size == 0
    lon, lat, grid, obs, DX, DY = _case(g, "a")
    d, r, c = ob.sparse_op_points(grid, obs, 1, ob.dmax_from_metrics(DX, DY, 1))
    assert d.size > 0 and np.all(d == 1.0)
