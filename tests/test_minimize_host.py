"""Host logic of the outer minimisation: the Moré-Thuente line search
restated in vardyn_gb300/minimize.py against scipy's own implementation of
the same MINPACK-2 algorithm (scipy.optimize._dcsrch.DCSRCH), on 1-D
functions that exercise every dcstep case."""
import numpy as np
import pytest

from vardyn_gb300.minimize import LineSearch

DCSRCH = pytest.importorskip("scipy.optimize._dcsrch").DCSRCH


def run_ours(phi, dphi, stp0, ftol, gtol, xtol, stpmax, maxiter=100):
    ls = LineSearch(ftol, gtol, xtol, 0.0, stpmax)
    f0, g0 = phi(0.0), dphi(0.0)
    task, stp = ls.start(f0, g0, stp0)
    n = 0
    trail = []
    while task.startswith("FG") and n < maxiter:
        f, g = phi(stp), dphi(stp)
        trail.append(stp)
        task, stp = ls.step(f, g, stp)
        n += 1
    return stp, task, trail


FUNCS = {
    # smooth convex with minimum near 0.73
    "quad": (lambda a: (a - 0.73) ** 2 - 0.5, lambda a: 2 * (a - 0.73)),
    # Moré-Thuente test function 1: -a / (a^2 + b)
    "mt1": (lambda a: -a / (a * a + 2.0), lambda a: (a * a - 2.0) / (a * a + 2.0) ** 2),
    # test function 2: (a + b)^5 - 2 (a + b)^4
    "mt2": (lambda a: (a + 0.004) ** 5 - 2 * (a + 0.004) ** 4,
            lambda a: 5 * (a + 0.004) ** 4 - 8 * (a + 0.004) ** 3),
    # oscillating: phi(a) = (1 - a) + 0.1 sin(10 pi a)... shifted to have g(0) < 0
    "osc": (lambda a: -a + 0.02 * np.sin(20 * a) + 0.5 * a * a,
            lambda a: -1 + 0.4 * np.cos(20 * a) + a),
}


@pytest.mark.parametrize("name", sorted(FUNCS))
@pytest.mark.parametrize("stp0", [1e-3, 0.1, 1.0, 10.0, 1000.0])
@pytest.mark.parametrize("tols", [(1e-3, 0.9, 0.1), (1e-4, 0.1, 1e-2)])
def test_line_search_matches_scipy(name, stp0, tols):
    phi, dphi = FUNCS[name]
    ftol, gtol, xtol = tols
    if dphi(0.0) >= 0:
        pytest.skip("ascent direction")
    stp, task, trail = run_ours(phi, dphi, stp0, ftol, gtol, xtol, 1e10)
    seen = []

    def sphi(a):
        seen.append(a)
        return phi(a)
    ref = DCSRCH(sphi, dphi, ftol, gtol, xtol, 0.0, 1e10)
    sstp, sphi1, sphi0, stask = ref(stp0, phi(0.0), dphi(0.0), maxiter=100)
    assert seen == trail
    if sstp is None:
        assert not task.startswith("CONV")
    else:
        assert stp == sstp
        assert task.startswith("CONV") == (stask[:4] == b"CONV" or str(stask).startswith("CONV"))

