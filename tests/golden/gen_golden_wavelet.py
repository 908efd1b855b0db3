"""Generate golden vectors for the wavelet reduced basis from the reference's
own ``mapping/src/basis.py`` (``Basis_wavelet3d``, 2640-2986, numpy form):
the number of coefficients, prior Q, and operg / operg_transpose on seeded
controls, on a lon/lat grid with land.

Under numpy 2, ``set_basis`` stops at basis.py:2800, where the size-1 array
that ``tools.gaspari_cohn`` returns for a scalar is stored into one element
of an array (numpy 1 stored its single value). The loaded module's
``gaspari_cohn`` is therefore wrapped to hand back that single value as a
0-d array for scalar arguments; the reference files are not modified.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_wavelet.py <VarDyn checkout>
Writes ``tests/golden/wavelet_golden.npz``.
"""
import os
import sys
from types import SimpleNamespace as NS

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

from gen_golden_basis import load_basis  # noqa: E402

WAV = dict(facnst=1.0, npsp=3.5, facpsp=1.5, lmin=60., lmax=250., tmin=3., tmax=15., sigma_Q=0.02)
TIMES_K = (0, 7, 21, 40)


def main():
    ref_root = _jax_standin.reference_root()
    basis = load_basis(ref_root)
    gc = basis.gaspari_cohn

    def gaspari_cohn_scalar(r, c):
        out = gc(r, c)
        return np.reshape(out, ()) if np.ndim(r) == 0 and np.size(out) == 1 else out
    basis.gaspari_cohn = gaspari_cohn_scalar
    lon1d = -65.0 + 0.1 * np.arange(40)
    lat1d = 33.0 + 0.1 * np.arange(30)
    lon, lat = np.meshgrid(lon1d, lat1d)
    ny, nx = lon.shape
    mask = np.zeros((ny, nx), dtype=bool)
    mask[8:15, 20:28] = True
    mask[-3:, :4] = True
    state = NS(ny=ny, nx=nx, lon=lon, lat=lat, mask=mask)
    cfg = NS(EXP=NS(tmp_DA_path="."), BASIS=NS(name_mod_var="ssh", path_background=None, var_background=None,
                                                **WAV))
    time = np.arange(0, 10.01, 0.25)
    W = basis.Basis_wavelet3d(cfg, state)
    _, Q = W.set_basis(time, return_q=True)
    out = dict(lon=lon1d, lat=lat1d, mask=mask, time=time, times_k=np.array(TIMES_K), q=np.asarray(Q),
               nbasis=np.int64(W.nbasis))
    rng = np.random.default_rng(57)
    X = rng.standard_normal(W.nbasis)
    out["X"] = X
    for k in TIMES_K:
        t = time[k]
        out[f"t{k}_phi"] = np.asarray(W.operg(t, X))
        ad = rng.standard_normal((ny, nx))
        out[f"t{k}_ad"] = ad
        out[f"t{k}_adX"] = np.asarray(W.operg_transpose(t, {"ssh": ad.copy()}))
    np.savez_compressed(os.path.join(HERE, "wavelet_golden.npz"), **out)
    print("wrote", len(out), "arrays, nbasis", W.nbasis)


if __name__ == "__main__":
    main()
