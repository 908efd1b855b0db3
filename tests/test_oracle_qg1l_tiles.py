"""The overlapping-tile QG 1.5-layer oracle (QgmWithTiles, jqgm.py:1033-1376)
against golden vectors produced by the reference's own jqgm.py source
(tests/golden/gen_golden_tiles.py)."""
import os

import numpy as np
import pytest

from oracle.qg1l_tiles import QgmTilesOracle, tile_origins

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qgt_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _close(a, b, tol):
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert np.array_equal(nan_a, nan_b)
    d = np.abs(a[~nan_a] - b[~nan_b]).max()
    return d <= tol * np.abs(b[~nan_b]).max()


def test_tiles_euler_land_mdt(g):
    o = QgmTilesOracle(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, Kdiffus=30.0, g=9.81,
                       f=1.0e-4, time_scheme="Euler", mdt=g["a_mdt"], tile_size=20, tile_overlap=6)
    assert np.array_equal(np.array(o.tiles), g["a_tiles"])
    assert np.abs(o.wsum - g["a_wsum"]).max() == 0.0
    assert _close(o.step(g["a_h0"], g["a_hb"], nstep=4), g["a_h1"], 1e-12)


def test_tiles_rk2_beta_plane_spatial_c(g):
    o = QgmTilesOracle(dx=g["b_dx"], dy=g["b_dy"], dt=900.0, SSH=g["b_ssh"], c=g["b_c"], Kdiffus=None, g=9.81,
                       f=g["b_f"], time_scheme="rk2", tile_size=16, tile_overlap=4)
    assert np.array_equal(np.array(o.tiles), g["b_tiles"])
    assert _close(o.step(g["b_ssh"], g["b_hb"], nstep=3), g["b_h1"], 1e-12)


def test_tile_origins_cover_the_domain():
    for ny, nx, T, ov in ((40, 52, 20, 6), (64, 64, 16, 4), (33, 70, 24, 8)):
        cov = np.zeros((ny, nx), int)
        for ys, xs in tile_origins(ny, nx, T, ov):
            assert 0 <= ys <= ny - T and 0 <= xs <= nx - T
            cov[ys:ys + T, xs:xs + T] += 1
        assert cov.min() >= 1


def _tl_case(scheme, seed):
    rng = np.random.default_rng(seed)
    ny, nx = 30, 38
    dx = np.full((ny, nx), 1.0e4)
    ssh = 0.1 * rng.standard_normal((ny, nx))
    ssh[12:15, 17:20] = np.nan
    hb = 0.01 * rng.standard_normal((ny, nx))
    hb[np.isnan(ssh)] = 0.0
    o = QgmTilesOracle(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=2.7, Kdiffus=20.0, f=1.0e-4, time_scheme=scheme,
                       tile_size=16, tile_overlap=4, mdt=0.02 * rng.standard_normal((ny, nx)))
    return o, np.nan_to_num(ssh), hb, rng


@pytest.mark.parametrize("scheme", ["Euler", "rk2"])
def test_tangent_matches_central_differences(scheme):
    o, h0, hb, rng = _tl_case(scheme, 3)
    d = 1e-3 * rng.standard_normal(h0.shape)
    tl = o.step_tgl(d, h0, hb, 3)
    eps = 1e-4     # the upwind switch makes larger steps cross kinks (1e-4 relative at 1e-3 for rk2)
    fd = (o.step(h0 + eps * d, hb, 3) - o.step(h0 - eps * d, hb, 3)) / (2 * eps)
    m = ~np.isnan(fd)
    assert np.all(tl[~m] == 0)
    assert np.abs(fd[m] - tl[m]).max() <= 1e-8 * np.abs(tl[m]).max()


@pytest.mark.parametrize("scheme", ["Euler", "rk2"])
def test_adjoint_dot_product(scheme):
    o, h0, hb, rng = _tl_case(scheme, 4)
    d = rng.standard_normal(h0.shape)
    y = rng.standard_normal(h0.shape)
    tl = o.step_tgl(d, h0, hb, 3)
    ad = o.step_adj(y, h0, hb, 3)
    lhs, rhs = float(np.sum(tl * y)), float(np.sum(d * ad))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
