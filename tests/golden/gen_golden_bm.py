"""Generate golden vectors for the wave-packet reduced basis from the
reference's own ``mapping/src/basis.py`` (``Basis_bm``, 472-937, numpy
form): frequencies, directions, per-frequency lattices and time centres,
prior Q, and operg / operg_transpose on seeded controls, on a lon/lat grid
with land.

The numpy form keeps a time centre while |dt| < tdec; the jax form
(``Basis_bm_jax``, 1026-1035) also keeps |dt| = tdec, whose weight
cos^2(pi/2) is below 1e-32: the two give the same fields to rounding.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_bm.py <VarDyn checkout>
Writes ``tests/golden/bm_golden.npz``.
"""
import datetime
import os
import sys
from types import SimpleNamespace as NS

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

from gen_golden_basis import load_basis  # noqa: E402

BM = dict(lmin=60., lmax=300., npsp=3.5, facpsp=1.5, lmeso=150., tmeso=10., facns=1.2, facnlt=2.0, tdecmin=2.,
          tdecmax=20., factdec=1., sloptdec=-1.28, Qmax=1e-3, slopQ=-2., norm_time=True, flux=False)
INIT_DATE = datetime.datetime(2012, 10, 1)
TIMES_K = (0, 9, 22, 40)


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
    cfg = NS(EXP=NS(init_date=INIT_DATE, tmp_DA_path="."),
             BASIS=NS(name_mod_var="ssh", file_depth=None, depth=None, name_var_depth=None, facQ=1,
                      compute_velocities=False, name_mod_u=None, name_mod_v=None, path_background=None,
                      var_background=None, **BM))
    time = np.arange(0, 10.01, 0.25)
    B = basis.Basis_bm(cfg, state)
    _, Q = B.set_basis(time, return_q=True)
    out = dict(lon=lon1d, lat=lat1d, mask=mask, time=time, times_k=np.array(TIMES_K),
               time_ref=np.float64(B.delta_time_ref), ff=np.asarray(B.ff), tdec=np.asarray(B.tdec, dtype=float),
               theta=np.asarray(B.theta), NP=np.asarray(B.NP), bounds=np.asarray(B.iff_wavebounds), q=np.asarray(Q))
    for iff in range(B.nf):
        out[f"f{iff}_lat"] = np.asarray(B.ENSLAT[iff], dtype=float)
        out[f"f{iff}_lon"] = np.asarray(B.ENSLON[iff], dtype=float)
        out[f"f{iff}_enst"] = np.asarray(B.enst[iff], dtype=float)
    rng = np.random.default_rng(91)
    X = rng.standard_normal(B.nbasis)
    out["X"] = X
    for k in TIMES_K:
        t = time[k]
        out[f"t{k}_phi"] = np.asarray(B.operg(t, X))
        ad = rng.standard_normal((ny, nx))
        out[f"t{k}_ad"] = ad
        out[f"t{k}_adX"] = np.asarray(B.operg_transpose(t, {"ssh": ad.copy()}))
    np.savez_compressed(os.path.join(HERE, "bm_golden.npz"), **out)
    print("wrote", len(out), "arrays, nbasis", B.nbasis, "nf", B.nf)


if __name__ == "__main__":
    main()
