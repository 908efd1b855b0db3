"""Generate golden vectors for the observation operators from the reference's
own ``mapping/src/obsop.py`` and ``mapping/src/grid.py``:

- ``Obsop_interp_l3`` (scipy form): the constructor's excluded border and
  mask points (obsop.py:118-134, via Obsop_interp.__init__) and
  ``_sparse_op`` (obsop.py:197-219), stored as (row, col, data) of H;
- ``Obsop_interp_l3_jax``: ``_sparse_op`` (KDTree, obsop.py:417-460).

Both run unmodified on a lon/lat grid with land, with and without masked
borders, for npix 4 and 1. jax is the NumPy stand-in of ``_jax_standin.py``;
the modules these code paths import but never call (xarray, pandas,
pyinterp, matplotlib, jax.experimental.sparse) are empty modules.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_obs.py <VarDyn checkout>
Writes ``tests/golden/obs_golden.npz``.
"""
import datetime
import importlib.util
import os
import sys
import types
from types import SimpleNamespace as NS

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402


def _empty(name):
    if name not in sys.modules:
        sys.modules[name] = types.ModuleType(name)
    return sys.modules[name]


def load_obsop(ref_root):
    _jax_standin.install(enable_x64=True)
    for name in ("xarray", "pandas", "pyinterp", "pyinterp.fill"):
        _empty(name)
    sys.modules["pyinterp"].fill = sys.modules["pyinterp.fill"]
    jax = sys.modules["jax"]
    exp = _empty("jax.experimental")
    exp.sparse = _empty("jax.experimental.sparse")
    jax.experimental = exp
    src_dir = os.path.join(ref_root, "mapping", "src")
    mods = {}
    for name in ("grid", "obsop"):
        spec = importlib.util.spec_from_file_location(f"src.{name}", os.path.join(src_dir, f"{name}.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"src.{name}"] = mod
        setattr(sys.modules["src"], name, mod)
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods["obsop"], mods["grid"]


def _objects(lon1d, lat1d, mask, npix, mask_borders):
    lon, lat = np.meshgrid(lon1d, lat1d)
    ny, nx = lon.shape
    dlon, dlat = lon1d[1] - lon1d[0], lat1d[1] - lat1d[0]
    DX = np.radians(dlon) * 6371e3 * np.cos(np.radians(lat))
    DY = np.full((ny, nx), np.radians(dlat) * 6371e3)
    state = NS(lon=lon, lat=lat, ny=ny, nx=nx, mask=mask, DX=DX, DY=DY, dx=float(DX.mean()), dy=float(DY.mean()),
               lon_min=lon.min(), lon_max=lon.max(), lat_min=lat.min(), lat_max=lat.max())
    config = NS(EXP=NS(lon_obs_max=None, lon_obs_min=None, lat_obs_max=None, lat_obs_min=None,
                       assimilation_time_step=datetime.timedelta(hours=1), tmp_DA_path="."),
                OBSOP=NS(compute_op=True, write_op=False, path_save=None, mask_borders=mask_borders, Npix=npix,
                         name_obs=None, name_var="SSH"))
    model = NS(name_var={"SSH": "ssh"}, timestamps=[], T=[], dt=3600.0)
    return config, state, model


def run_case(obsop, tag, out, mask_borders, seed):
    rng = np.random.default_rng(seed)
    lon1d = -70.0 + 0.05 * np.arange(36)
    lat1d = 30.0 + 0.05 * np.arange(28)
    ny, nx = lat1d.size, lon1d.size
    mask = np.zeros((ny, nx), dtype=bool)
    mask[10:14, 12:17] = True
    mask[20:, 3] = True
    nobs = 400
    lon_obs = rng.uniform(lon1d[0] - 0.08, lon1d[-1] + 0.08, nobs)
    lat_obs = rng.uniform(lat1d[0] - 0.08, lat1d[-1] + 0.08, nobs)
    out.update({f"{tag}_lon": lon1d, f"{tag}_lat": lat1d, f"{tag}_mask": mask, f"{tag}_lon_obs": lon_obs,
                f"{tag}_lat_obs": lat_obs})
    for npix in (4, 1):
        config, state, model = _objects(lon1d, lat1d, mask, npix, mask_borders)
        op = obsop.Obsop_interp_l3(config, state, {}, model)
        H = op._sparse_op(lon_obs, lat_obs).tocoo()
        order = np.lexsort((H.col, H.row))
        out[f"{tag}_l3_n{npix}_row"] = np.asarray(H.row)[order].astype(np.int64)
        out[f"{tag}_l3_n{npix}_col"] = np.asarray(H.col)[order].astype(np.int64)
        out[f"{tag}_l3_n{npix}_data"] = np.asarray(H.data)[order]
        out[f"{tag}_dmax_n{npix}"] = np.float64(op.dmax)
        if npix == 4:
            out[f"{tag}_ind_mask"] = np.asarray(op.ind_mask, dtype=np.int64)
            out[f"{tag}_ind_borders"] = np.asarray(op.ind_borders, dtype=np.int64)
        opj = obsop.Obsop_interp_l3_jax(config, state, {}, model)
        data, indices = opj._sparse_op(lon_obs, lat_obs)
        out[f"{tag}_jax_n{npix}_data"] = np.asarray(data, dtype=np.float64)
        out[f"{tag}_jax_n{npix}_indices"] = np.asarray(indices, dtype=np.int64)


def main():
    ref_root = _jax_standin.reference_root()
    obsop, grid = load_obsop(ref_root)
    out = {}
    run_case(obsop, "a", out, mask_borders=False, seed=31)
    run_case(obsop, "b", out, mask_borders=True, seed=32)
    pts = np.array([[-70.0, 30.0], [-68.3, 31.2], [10.0, -45.0]])
    out["geo2cart_in"] = pts
    out["geo2cart_out"] = np.asarray(grid.geo2cart(pts))
    np.savez_compressed(os.path.join(HERE, "obs_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
