"""The wavelet reduced basis against golden vectors produced by the
reference's own basis.py (Basis_wavelet3d, tests/golden/gen_golden_wavelet.py):
the library's coefficient count and Q, and the oracle's G and G^T, on a
lon/lat grid with land."""
import os

import numpy as np
import pytest

from oracle.basis import WaveletOracle
from vardyn_gb300.basis import WaveletParams, WaveletPlan

GOLD = os.path.join(os.path.dirname(__file__), "golden", "wavelet_golden.npz")
WAV = dict(facnst=1.0, npsp=3.5, facpsp=1.5, lmin=60., lmax=250., tmin=3., tmax=15., sigma_Q=0.02)


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def test_library_host_tables_match_reference(g):
    pl = WaveletPlan(g["lon"], g["lat"], g["time"], WaveletParams(**WAV), land=g["mask"], geographic=True,
                     host_only=True)
    assert pl.nbasis == int(g["nbasis"])
    assert np.array_equal(pl.q(), g["q"])


def test_oracle_projection_and_transpose_match_reference(g):
    lon, lat = np.meshgrid(g["lon"], g["lat"])
    o = WaveletOracle(lon, lat, mask=g["mask"], geo=True, **WAV)
    _, Q = o.set_basis(g["time"])
    assert np.array_equal(Q, g["q"])
    for k in g["times_k"]:
        t = g["time"][k]
        phi, want = o.operg(t, g["X"]), g[f"t{k}_phi"]
        assert np.abs(want).max() > 0 and np.abs(phi - want).max() <= 1e-13 * np.abs(want).max()
        adX, want_ad = o.operg_transpose(t, g[f"t{k}_ad"]), g[f"t{k}_adX"]
        assert np.abs(adX - want_ad).max() <= 1e-13 * np.abs(want_ad).max()
