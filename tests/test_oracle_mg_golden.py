"""The masked multigrid Helmholtz restatement (oracle/helmholtz_mg.py)
against golden solutions produced by the reference's own
helmholtz_multigrid.py (tests/golden/gen_golden_mg.py): exact bottom solve,
bottom smoothing, and a single-level grid."""
import os

import numpy as np
import pytest

from oracle.helmholtz_mg import MGOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "mg_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


@pytest.mark.parametrize("t", ["a", "b", "c"])
def test_oracle_solve_matches_reference(g, t):
    nx, ny, nb, ite, nlev = (int(v) for v in g[f"{t}_meta"])
    o = MGOracle(1.0, 1.3, nx, ny, g[f"{t}_cu"], g[f"{t}_cv"], g[f"{t}_lam"], mask=g[f"{t}_mask"],
                 niter_bottom=nb, max_ite=ite)
    assert o.n_levels == nlev
    f = o.solve(g[f"{t}_rhs"])
    want = g[f"{t}_f"]
    assert np.abs(f - want).max() <= 1e-12 * np.abs(want).max()
