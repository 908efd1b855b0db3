"""Generate golden vectors for the Gaussian space-time reduced basis from the
reference's own ``mapping/src/basis.py`` (``Basis_gauss3d``, 1170-1555):
lattice (ENST, ENSLAT, ENSLON), prior Q, active time weights, and operg /
operg_transpose on seeded controls, for three components on a lon/lat grid
with land (default, with spin-up, flux window without normalisation).
``Basis_multi`` (4039-4136) concatenates its components' controls and sums
their fields, so the components pin it too.

jax is the NumPy stand-in of ``_jax_standin.py``; the modules these code
paths import but never call (xarray, pyinterp, netCDF4,
jax.experimental.sparse) are empty modules.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_basis.py <VarDyn checkout>
Writes ``tests/golden/basis_golden.npz``.
"""
import importlib.util
import os
import sys
from types import SimpleNamespace as NS

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

from gen_golden_obs import _empty, load_obsop  # noqa: E402

COMPS = [dict(sigma_D=100.0, sigma_T=5.0, facns=2.0, facnlt=2.0, sigma_Q=0.1, normalize_fact=True, flux=False,
              time_spinup=None),
         dict(sigma_D=60.0, sigma_T=10.0, facns=1.5, facnlt=3.0, sigma_Q=0.2, normalize_fact=True, flux=False,
              time_spinup=3.0),
         dict(sigma_D=80.0, sigma_T=4.0, facns=1.0, facnlt=1.0, sigma_Q=0.3, normalize_fact=False, flux=True,
              time_spinup=None)]
TIMES_K = (0, 5, 17, 40)


def load_basis(ref_root):
    load_obsop(ref_root)                      # stand-ins, src.grid
    sys.modules["netCDF4"] = _empty("netCDF4")
    sys.modules["netCDF4"].Dataset = None
    src_dir = os.path.join(ref_root, "mapping", "src")
    for name in ("tools", "basis"):
        spec = importlib.util.spec_from_file_location(f"src.{name}", os.path.join(src_dir, f"{name}.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"src.{name}"] = mod
        setattr(sys.modules["src"], name, mod)
        spec.loader.exec_module(mod)
    return sys.modules["src.basis"]


def main():
    ref_root = _jax_standin.reference_root()
    basis = load_basis(ref_root)
    lon1d = -65.0 + 0.1 * np.arange(40)
    lat1d = 33.0 + 0.1 * np.arange(30)
    lon, lat = np.meshgrid(lon1d, lat1d)
    ny, nx = lon.shape
    mask = np.zeros((ny, nx), dtype=bool)
    mask[8:15, 20:28] = True
    mask[-3:, :4] = True
    DX = np.radians(0.1) * 6371e3 * np.cos(np.radians(lat))
    DY = np.full((ny, nx), np.radians(0.1) * 6371e3)
    state = NS(ny=ny, nx=nx, lon=lon, lat=lat, lon_min=lon.min(), lon_max=lon.max(), lat_min=lat.min(),
               lat_max=lat.max(), f=np.full((ny, nx), 1e-4), DX=DX, DY=DY, mask=mask, lon_unit="-180_180")
    time = np.arange(0, 10.01, 0.25)
    out = dict(lon=lon1d, lat=lat1d, mask=mask, time=time, times_k=np.array(TIMES_K))
    rng = np.random.default_rng(77)
    ads = {k: rng.standard_normal((ny, nx)) for k in TIMES_K}    # one cotangent per time, shared by components
    for k in TIMES_K:
        out[f"t{k}_ad"] = ads[k]
    for c, p in enumerate(COMPS):
        cfg = NS(BASIS=NS(name_mod_var="ssh", fcor=None, flag_variable_Q=False, path_sad=None, name_var_sad=None,
                          path_background=None, var_background=None, c_grid_var=None, compute_velocities=False,
                          name_mod_u=None, name_mod_v=None, **p))
        B = basis.Basis_gauss3d(cfg, state)
        _, Q = B.set_basis(time, return_q=True)
        out[f"c{c}_enst"], out[f"c{c}_enslat"], out[f"c{c}_enslon"] = B.ENST, B.ENSLAT, B.ENSLON
        out[f"c{c}_q"] = np.asarray(Q)
        X = rng.standard_normal(B.nbasis)
        out[f"c{c}_X"] = X
        for k in TIMES_K:
            t = time[k]
            g = B.Gauss_t[t]
            nz = np.nonzero(g)[0]
            out[f"c{c}_t{k}_gt_idx"], out[f"c{c}_t{k}_gt_val"] = nz, g[nz]
            out[f"c{c}_t{k}_phi"] = np.asarray(B.operg(t, X))
            out[f"c{c}_t{k}_adX"] = np.asarray(B.operg_transpose(t, {"ssh": ads[k].copy()}))
    np.savez_compressed(os.path.join(HERE, "basis_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
