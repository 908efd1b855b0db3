"""The Gaussian reduced basis against golden vectors produced by the
reference's own basis.py (tests/golden/gen_golden_basis.py): the library's
host tables (lattice, Q, time weights) and the oracle's G and G^T, three
components on a lon/lat grid with land."""
import os

import numpy as np
import pytest

from oracle.basis import Gauss3dOracle
from vardyn_gb300.basis import BasisPlan, Gauss3dParams

GOLD = os.path.join(os.path.dirname(__file__), "golden", "basis_golden.npz")
COMPS = [dict(sigma_D=100.0, sigma_T=5.0, facns=2.0, facnlt=2.0, sigma_Q=0.1, normalize_fact=True, flux=False,
              time_spinup=None),
         dict(sigma_D=60.0, sigma_T=10.0, facns=1.5, facnlt=3.0, sigma_Q=0.2, normalize_fact=True, flux=False,
              time_spinup=3.0),
         dict(sigma_D=80.0, sigma_T=4.0, facns=1.0, facnlt=1.0, sigma_Q=0.3, normalize_fact=False, flux=True,
              time_spinup=None)]


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _close(a, b, tol):
    return np.abs(np.asarray(a) - b).max() <= tol * max(np.abs(b).max(), 1e-300)


def test_library_host_tables_match_reference(g):
    plan = BasisPlan(g["lon"], g["lat"], g["time"], [Gauss3dParams(**c) for c in COMPS], land=g["mask"],
                     geographic=True, host_only=True)
    q = plan.q()
    for c in range(len(COMPS)):
        off, nt, ns = plan.component(c)
        enst, lat, lon = plan.lattice(c)
        assert (nt, ns) == (g[f"c{c}_enst"].size, g[f"c{c}_enslat"].size)
        assert _close(enst, g[f"c{c}_enst"], 1e-14) and _close(lat, g[f"c{c}_enslat"], 1e-14)
        assert _close(lon, g[f"c{c}_enslon"], 1e-14)
        assert _close(q[off:off + nt * ns], g[f"c{c}_q"], 1e-15)
        for k in g["times_k"]:
            idx, val = g[f"c{c}_t{k}_gt_idx"], g[f"c{c}_t{k}_gt_val"]
            want = sorted({(int(i) // ns, float(v)) for i, v in zip(idx, val)})
            got = sorted(plan.time_weights(int(k), c))
            assert [i for i, _ in got] == [i for i, _ in want]
            assert np.allclose([w for _, w in got], [w for _, w in want], rtol=1e-14, atol=0)


@pytest.mark.parametrize("c", range(len(COMPS)))
def test_oracle_projection_and_transpose_match_reference(g, c):
    lon, lat = np.meshgrid(g["lon"], g["lat"])
    o = Gauss3dOracle(lon, lat, mask=g["mask"], geo=True, **COMPS[c])
    o.set_basis(g["time"])
    assert np.array_equal(o.ENST, g[f"c{c}_enst"]) and np.array_equal(o.ENSLAT, g[f"c{c}_enslat"])
    assert np.array_equal(o.ENSLON, g[f"c{c}_enslon"])
    for k in g["times_k"]:
        t = g["time"][k]
        assert _close(o.operg(t, g[f"c{c}_X"]), g[f"c{c}_t{k}_phi"], 1e-13)
        assert _close(o.operg_transpose(t, g[f"t{k}_ad"]), g[f"c{c}_t{k}_adX"], 1e-13)
