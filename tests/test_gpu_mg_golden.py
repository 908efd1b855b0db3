"""The library's multigrid Helmholtz solver (drop-in MG_Helmholtz, vd_mg_*)
against golden solutions produced by the reference's own
helmholtz_multigrid.py (tests/golden/gen_golden_mg.py)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "mg_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.mark.parametrize("t", ["a", "b", "c"])
def test_library_solve_matches_reference(t):
    import torch
    from vardyn_gb300.helmholtz_mg import MG_Helmholtz
    g = dict(np.load(GOLD))
    nx, ny, nb, ite, nlev = (int(v) for v in g[f"{t}_meta"])
    s = MG_Helmholtz(1.0, 1.3, nx, ny, g[f"{t}_cu"], g[f"{t}_cv"], lambd=g[f"{t}_lam"], mask=g[f"{t}_mask"],
                     niter_bottom=nb, max_ite=ite)
    assert s.n_levels == nlev
    f = s.solve(g[f"{t}_rhs"])
    f = f.cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
    want = g[f"{t}_f"]
    assert np.abs(f - want).max() <= 1e-11 * np.abs(want).max()
