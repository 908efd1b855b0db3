"""Overlapping-tile QG 1.5-layer model on the GPU (vd_qgt_step, drop-in
QgmWithTiles.step) against the reference's own QgmWithTiles outputs
(tests/golden/gen_golden_tiles.py) and the float64 oracle."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qgt_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _rel(a, b):
    m = ~np.isnan(b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    return float(np.abs(a[m] - b[m]).max() / np.abs(b[m]).max())


def test_euler_land_mdt_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import QgmWithTiles
    m = QgmWithTiles(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, Kdiffus=30.0, g=9.81, f=1.0e-4,
                     time_scheme="Euler", mdt=g["a_mdt"], tile_size=20, tile_overlap=6, dtype="float64")
    assert np.array_equal(np.array(m.tiles), g["a_tiles"])
    assert _rel(m.step(g["a_h0"], g["a_hb"], nstep=4), g["a_h1"]) < 1e-11


def test_rk2_beta_plane_spatial_c_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import QgmWithTiles
    m = QgmWithTiles(dx=g["b_dx"], dy=g["b_dy"], dt=900.0, SSH=g["b_ssh"], c=g["b_c"], Kdiffus=None, g=9.81,
                     f=g["b_f"], time_scheme="rk2", tile_size=16, tile_overlap=4, dtype="float64")
    assert _rel(m.step(g["b_ssh"], g["b_hb"], nstep=3), g["b_h1"]) < 1e-11


def _case(ny, nx, seed, land=True):
    rng = np.random.default_rng(seed)
    dx = np.full((ny, nx), 5.0e3)
    ssh = 0.1 * rng.standard_normal((ny, nx))
    if land:
        ssh[ny // 3:ny // 3 + 5, nx // 2:nx // 2 + 6] = np.nan
    hb = 0.01 * rng.standard_normal((ny, nx))
    hb[np.isnan(ssh)] = 0.0
    return dx, ssh, hb


def test_float64_tile32_matches_oracle():
    from oracle.qg1l_tiles import QgmTilesOracle
    from vardyn_gb300.model_qg1l.jqgm import QgmWithTiles
    dx, ssh, hb = _case(70, 90, 3)
    kw = dict(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=2.7, Kdiffus=20.0, g=9.81, f=1.0e-4, time_scheme="rk2",
              tile_size=32, tile_overlap=8)
    h0 = np.nan_to_num(ssh)
    ref = QgmTilesOracle(**kw).step(h0, hb, nstep=5)
    got = QgmWithTiles(dtype="float64", **kw).step(h0, hb, nstep=5)
    assert _rel(got, ref) < 1e-11


def test_float32_default_tile_matches_oracle():
    """The reference's default tiles (64, overlap 8) in float32."""
    from oracle.qg1l_tiles import QgmTilesOracle
    from vardyn_gb300.model_qg1l.jqgm import QgmWithTiles
    dx, ssh, hb = _case(160, 192, 4)
    kw = dict(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=2.7, Kdiffus=None, g=9.81, f=1.0e-4, time_scheme="Euler",
              tile_size=64, tile_overlap=8)
    h0 = np.nan_to_num(ssh)
    ref = QgmTilesOracle(**kw).step(h0, hb, nstep=4)
    got = QgmWithTiles(dtype="float32", **kw).step(h0, hb, nstep=4)
    m = ~np.isnan(ref)
    err = np.linalg.norm(got[m] - ref[m]) / np.linalg.norm(ref[m])
    print(f"QgmWithTiles float32 rel-L2 vs float64 oracle: {err:.2e}")
    assert err < 1e-5


def test_guards():
    from vardyn_gb300.model_qg1l.jqgm import QgmWithTiles
    dx, ssh, hb = _case(80, 80, 5, land=False)
    with pytest.raises(ValueError):
        QgmWithTiles(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=2.7, f=1e-4, tile_size=64, dtype="float64")
    with pytest.raises(ValueError):
        QgmWithTiles(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=2.7, f=1e-4, time_scheme="rk3", tile_size=32)
    m = QgmWithTiles(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=2.7, f=1e-4, tile_size=32, tile_overlap=8)
    with pytest.raises(NotImplementedError):
        m.step_adj(hb, ssh, hb, 1)
