"""The wave-packet reduced basis against golden vectors produced by the
reference's own basis.py (Basis_bm, tests/golden/gen_golden_bm.py): the
library's host tables (frequencies, decorrelation times, directions,
lattices, time centres, Q) and the oracle's G and G^T, on a lon/lat grid
with land."""
import os

import numpy as np
import pytest

from oracle.basis import BMOracle
from vardyn_gb300.basis import BMParams, BMPlan

GOLD = os.path.join(os.path.dirname(__file__), "golden", "bm_golden.npz")
BM = dict(lmin=60., lmax=300., npsp=3.5, facpsp=1.5, lmeso=150., tmeso=10., facns=1.2, facnlt=2.0, tdecmin=2.,
          tdecmax=20., factdec=1., sloptdec=-1.28, Qmax=1e-3, slopQ=-2., norm_time=True, flux=False)


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _close(a, b, tol):
    b = np.asarray(b, dtype=float)
    return np.asarray(a).shape == b.shape and np.abs(np.asarray(a) - b).max() <= tol * max(np.abs(b).max(), 1e-300)


def test_library_host_tables_match_reference(g):
    plan = BMPlan(g["lon"], g["lat"], g["time"], BMParams(time_ref=float(g["time_ref"]), **BM), land=g["mask"],
                  geographic=True, host_only=True)
    assert plan.nf == g["ff"].size and plan.ntheta == g["theta"].size
    assert _close(plan.theta, g["theta"], 1e-15)
    assert _close(plan.q(), g["q"], 1e-15)
    for iff in range(plan.nf):
        ff, td, off, nt, ns = plan.frequency(iff)
        assert abs(ff - g["ff"][iff]) <= 1e-15 * g["ff"][iff] and abs(td - g["tdec"][iff]) <= 1e-14 * g["tdec"][iff]
        assert off == g["bounds"][iff] and ns == g["NP"][iff] and nt == g[f"f{iff}_enst"].size
        enst, lat, lon = plan.lattice(iff)
        assert _close(enst, g[f"f{iff}_enst"], 1e-13)
        assert _close(lat, g[f"f{iff}_lat"], 1e-14) and _close(lon, g[f"f{iff}_lon"], 1e-14)


def test_oracle_projection_and_transpose_match_reference(g):
    lon, lat = np.meshgrid(g["lon"], g["lat"])
    o = BMOracle(lon, lat, mask=g["mask"], geo=True, time_ref=float(g["time_ref"]), **BM)
    _, Q = o.set_basis(g["time"])
    assert _close(Q, g["q"], 1e-15)
    for k in g["times_k"]:
        t = g["time"][k]
        assert _close(o.operg(t, g["X"]), g[f"t{k}_phi"], 1e-13)
        assert _close(o.operg_transpose(t, g[f"t{k}_ad"]), g[f"t{k}_adX"], 1e-13)
