"""The oracle's spectral barotropic filter of the shallow-water model
(sw.py:305-320, 695-725; the DCT-II Neumann Helmholtz solver,
helmholtz.py:20-87, 187-305) against outputs of the reference's own sw.py and
helmholtz.py (tests/golden/gen_golden_swfilter.py): the solver's eigenvalues,
one solve, the right-hand side with the filter and a 3-step run. The
reference's solver does not construct with land (helmholtz.py:254), so the
case has none, and the oracle refuses land."""
import os

import numpy as np
import pytest

from oracle.sw import SWOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "swfilter_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _param(g, **over):
    p = "fa_"
    d = dict(nx=24, ny=20, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
             taux=0.05, tauy=-0.03, bottom_drag_coef=1e-6, dt=30.0, slip_coef=0.5, visc_coef=10.0, diff_coef=5.0,
             barotropic_filter=True, barotropic_filter_spectral=True)
    d.update(over)
    return d


def rel(a, b):
    return np.abs(np.asarray(a) - b).max() / np.abs(b).max()


def test_solver_eigenvalues_and_solve(g):
    o = SWOracle(_param(g))
    assert rel(o.helm_dct, g["fa_helm_dct"]) < 1e-14
    assert rel(o.neumann_solve(g["fa_rhs"]), g["fa_sol"]) < 1e-12


def test_rhs_with_filter(g):
    o = SWOracle(_param(g))
    u, v, h = o.to_model(g["fa_u0"], g["fa_v0"], g["fa_h0"])
    du, dv, dh = o.rhs(u, v, h, o.ref_values(o.H), o.taux, o.tauy)
    assert rel(du, g["fa_dtu"]) < 1e-12 and rel(dv, g["fa_dtv"]) < 1e-12 and rel(dh, g["fa_dth"]) < 1e-13
    # the filter changes the momentum tendencies (not a no-op on this case)
    o0 = SWOracle(_param(g, barotropic_filter=False))
    du0, _, _ = o0.rhs(u, v, h, o0.ref_values(o0.H), o0.taux, o0.tauy)
    assert rel(du0, g["fa_dtu"]) > 1e-3


def test_steps_with_filter(g):
    o = SWOracle(_param(g))
    r = o.step(g["fa_u0"], g["fa_v0"], g["fa_h0"], nstep=3)
    for a, k in zip(r, ["u3", "v3", "h3"]):
        assert rel(a, g["fa_" + k]) < 1e-12, k


def test_refused_forms(g):
    with pytest.raises(NotImplementedError):
        SWOracle(_param(g, barotropic_filter_spectral=False))
    mask = np.ones((24, 20))
    mask[8:12, 7:11] = 0
    with pytest.raises(NotImplementedError):
        SWOracle(_param(g, mask=mask))
