"""Generate golden vectors for the wave-packet basis with auxiliary
decorrelation times and variances from the reference's own
``mapping/src/basis.py`` (``Basis_bmaux``, 1741-2393, numpy form): per
frequency the lattice, per-centre decorrelation times, window integrals and
time centres, the prior Q, the space operators Gx and the time operators
Gt, on a lon/lat grid with land.

The auxiliary fields come from a NetCDF file in the reference
(``xr.open_dataset(file_aux)``, 1943-1950). xarray is not installed here, so
a small in-memory stand-in serves the calls the class makes: ``['lon'].data``,
``assign_coords``, ``sortby`` and ``DataArray.interp(f=, lon=, lat=)``. The
stand-in's ``interp`` follows xarray's rules for 1-D indexers: orthogonal
(outer-product) points, linear along each dimension in turn, NaN outside
the coordinates; it is written as successive 1-D interpolations, not with
the oracle's multilinear interpolator.

The numpy ``operg`` of the class accumulates the projection into a variable
it never returns (basis.py:2303-2320), so the projection vectors are formed
here from the reference's own Gx and Gt with the jax class's formula
(``Basis_bmaux_jax._operg``, 2473-2498: phi = sum_f Gx_f sum_it (Gt X)_f)
and its transpose.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_bmaux.py <VarDyn checkout>
Writes ``tests/golden/bmaux_golden.npz``.
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

BMAUX = dict(lmin=60., lmax=300., npsp=3.5, facpsp=1.5, facns=1.2, facnlt=2.0, tdecmin=2., tdecmax=15.,
             factdec=1.3, facQ=2.0, norm_time=True, flux=False)
INIT_DATE = datetime.datetime(2012, 10, 1)
TIMES_K = (0, 9, 22, 40)


def _lin1d(c, x):
    """(i0, w) with x = (1 - w) c[i0] + w c[i0 + 1]; i0 = -1 outside."""
    c = np.asarray(c, float)
    x = np.atleast_1d(np.asarray(x, float))
    i0 = np.searchsorted(c, x, side="right") - 1
    i0 = np.where(x == c[-1], len(c) - 2, i0)
    out = (x < c[0]) | (x > c[-1])
    i0 = np.clip(i0, 0, len(c) - 2)
    w = (x - c[i0]) / (c[i0 + 1] - c[i0])
    return np.where(out, -1, i0), w


class _DA:
    def __init__(self, values, coords):
        self.values = np.asarray(values)
        self.data = self.values
        self.coords = coords          # dict name -> 1-D array, in dimension order

    def min(self):
        return self.values.min()

    def interp(self, f, lon, lat):
        """Orthogonal linear interpolation of a (f, lat, lon) field, one
        dimension at a time: f (a scalar), then lat, then lon; NaN outside
        the coordinates. Result [lat][lon]."""
        c = self.coords

        def along(v, coord, x, axis):
            i0, w = _lin1d(coord, x)
            lo = np.take(v, np.maximum(i0, 0), axis=axis)
            hi = np.take(v, np.maximum(i0, 0) + 1, axis=axis)
            shape = [1] * v.ndim
            shape[axis] = len(w)
            r = (1 - w.reshape(shape)) * lo + w.reshape(shape) * hi
            return np.where((i0 < 0).reshape(shape), np.nan, r)

        v = along(self.values, c["f"], f, 0)[0]          # [lat][lon]
        v = along(v, c["lat"], lat, 0)                    # [nq_lat][lon]
        v = along(v, c["lon"], lon, 1)                    # [nq_lat][nq_lon]
        return _DA(v, {})


class _DS:
    def __init__(self, f, lat, lon, fields):
        self.f, self.lat, self.lon = np.asarray(f, float), np.asarray(lat, float), np.asarray(lon, float)
        self.fields = fields

    def __getitem__(self, key):
        if key == "lon":
            return _DA(self.lon, {})
        return _DA(self.fields[key], {"f": self.f, "lat": self.lat, "lon": self.lon})

    def assign_coords(self, d):
        (_, arr), = d.values()
        return _DS(self.f, self.lat, np.asarray(arr, float), self.fields)

    def sortby(self, da):
        order = np.argsort(self.lon, kind="stable")
        return _DS(self.f, self.lat, self.lon[order], {k: v[..., order] for k, v in self.fields.items()})


def aux_fields(seed=501):
    """Smooth synthetic Tdec [days] and Std [m] on (f, lat, lon); the lon
    axis is given unsorted to exercise the reference's sortby."""
    rng = np.random.default_rng(seed)
    fc = np.array([1 / 400., 1 / 200., 1 / 100., 1 / 40.])
    latc = np.linspace(32.2, 36.6, 12)
    lonc = np.linspace(-66.0, -60.3, 14)
    F, LA, LO = np.meshgrid(fc, latc, lonc, indexing="ij")
    tdec = 4.0 + 6.0 * np.exp(-((LA - 34.0) ** 2 + (LO + 63.0) ** 2) / 4.0) + 30.0 * F + \
        0.5 * rng.standard_normal(F.shape)
    std = 0.02 + 0.03 * np.exp(-((LA - 35.0) ** 2) / 3.0) * (1 + 20 * F) + 0.002 * rng.random(F.shape)
    perm = rng.permutation(lonc.size)
    return fc, latc, lonc[perm], tdec[..., perm], std[..., perm]


def main():
    ref_root = _jax_standin.reference_root()
    basis = load_basis(ref_root)
    fc, latc, lonc, tdec, std = aux_fields()
    ds = _DS(fc, latc, lonc, {"Tdec": tdec, "Std": std})
    basis.xr = NS(open_dataset=lambda *a, **k: ds)
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
             BASIS=NS(name_mod_var="ssh", file_aux="aux.nc", file_depth=None, name_var_depth=None,
                      file_facQaux=None, name_var_facQaux=None, facQ_aux_path=None, l_largescale=None,
                      facQ_largescale=None, compute_velocities=False, name_mod_u=None, name_mod_v=None,
                      path_background=None, var_background=None, **BMAUX))
    time = np.arange(0, 10.01, 0.25)
    B = basis.Basis_bmaux(cfg, state)
    _, Q = B.set_basis(time, return_q=True)
    out = dict(lon=lon1d, lat=lat1d, mask=mask, time=time, times_k=np.array(TIMES_K),
               time_ref=np.float64(B.delta_time_ref), ff=np.asarray(B.ff), theta=np.asarray(B.theta),
               NP=np.asarray(B.NP), bounds=np.asarray(B.iff_wavebounds), q=np.asarray(Q),
               aux_f=fc, aux_lat=latc, aux_lon=lonc, aux_tdec=tdec, aux_std=std)
    for iff in range(B.nf):
        out[f"f{iff}_lat"] = np.asarray(B.ENSLAT[iff], dtype=float)
        out[f"f{iff}_lon"] = np.asarray(B.ENSLON[iff], dtype=float)
        out[f"f{iff}_enst"] = np.asarray(B.enst[iff], dtype=float)
        out[f"f{iff}_tdec"] = np.asarray(B.tdec[iff], dtype=float)
        out[f"f{iff}_norm"] = np.asarray(B.norm_fact[iff], dtype=float)
    rng = np.random.default_rng(92)
    X = rng.standard_normal(B.nbasis)
    out["X"] = X
    for k in TIMES_K:
        t = time[k]
        phi = np.zeros(B.nphys)
        adX = np.zeros(B.nbasis)
        ad = rng.standard_normal((ny, nx))
        for iff in range(B.nf):
            lo, hi = B.iff_wavebounds[iff], B.iff_wavebounds[iff + 1]
            g = np.asarray(B.Gt[t][iff])
            nit = (hi - lo) // B.Nx[iff] if B.Nx[iff] else 0
            if nit == 0:
                continue
            phi += B.Gx[iff].dot((g * X[lo:hi]).reshape(nit, B.Nx[iff]).sum(axis=0))
            adX[lo:hi] = (g.reshape(nit, B.Nx[iff]) * B.Gx[iff].T.dot(ad.ravel())[None, :]).ravel()
        out[f"t{k}_phi"] = phi.reshape(ny, nx)
        out[f"t{k}_ad"] = ad
        out[f"t{k}_adX"] = adX
    np.savez_compressed(os.path.join(HERE, "bmaux_golden.npz"), **out)
    print("wrote", len(out), "arrays, nbasis", B.nbasis, "nf", B.nf, "NP", list(B.NP))


if __name__ == "__main__":
    main()
