"""The QG 1.5-layer model with tracers (Qgm_trac, jqgm.py:1551-2151) restated
in oracle/qg1l_trac.py against golden vectors produced by the reference's own
jqgm.py source (tests/golden/gen_golden_trac.py)."""
import os

import numpy as np
import pytest

from oracle.qg1l_trac import QgmTracOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qgtrac_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _rel(a, b):
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(b)
    return float(np.abs(a[m] - b[m]).max() / np.abs(b[m]).max())


def test_euler_two_tracers_open_boundaries(g):
    o = QgmTracOracle(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                      time_scheme="Euler", Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC", mdt=g["a_mdt"])
    assert _rel(o.step(g["a_X0"], g["a_Xb"], nstep=4), g["a_X1"]) < 1e-12


def test_rk2_dirichlet_relaxation_no_pv_advection(g):
    o = QgmTracOracle(dx=g["b_dx"], dy=g["b_dx"], dt=600.0, SSH=g["b_ssh"], c=2.5, g=9.81, f=1.0e-4,
                      time_scheme="rk2", Wbc=g["b_wbc"], Kdiffus=None, Kdiffus_trac=5.0, bc_trac="dirichlet",
                      advect_pv=False)
    assert _rel(o.step(g["b_X0"], g["b_Xb"], nstep=3), g["b_X1"]) < 1e-12


def test_rk2_without_tracers(g):
    o = QgmTracOracle(dx=g["c_dx"], dy=g["c_dx"], dt=900.0, SSH=g["c_ssh"], c=2.7, g=9.81, f=1.0e-4,
                      time_scheme="rk2", Kdiffus=15.0)
    assert _rel(o.step(g["c_ssh"], g["c_hb"], nstep=3), g["c_h1"]) < 1e-12


@pytest.mark.parametrize("change", [dict(bc_trac="OBC"), dict(Wbc=None), dict(Kdiffus_trac=None)])
def test_fixtures_tell_the_options_apart(g, change):
    kw = dict(dx=g["b_dx"], dy=g["b_dx"], dt=600.0, SSH=g["b_ssh"], c=2.5, g=9.81, f=1.0e-4, time_scheme="rk2",
              Wbc=g["b_wbc"], Kdiffus_trac=5.0, bc_trac="dirichlet", advect_pv=False)
    kw.update(change)
    assert _rel(QgmTracOracle(**kw).step(g["b_X0"], g["b_Xb"], nstep=3), g["b_X1"]) > 1e-6


def test_unknown_scheme_is_refused():
    with pytest.raises(ValueError):
        QgmTracOracle(dx=np.full((8, 8), 1e4), dy=np.full((8, 8), 1e4), dt=900.0, SSH=np.zeros((8, 8)), c=2.7,
                      time_scheme="rk3")


def test_rk4_extension_is_fourth_order():
    """The classical RK4 extension converges at fourth order in dt (error
    ratio 16 per halving), rk2 at second order (ratio 4). The flow is an
    eddy on a uniform current, so that no velocity changes sign: the upwind
    split max(u, 0) has a kink at u = 0 that lowers the order of any
    Runge-Kutta scheme."""
    ny, nx, d = 30, 34, 1.0e4
    jj, ii = np.mgrid[0:ny, 0:nx]
    ssh = 0.5e-6 * d * (ii - jj) + 0.01 * np.exp(-(((ii - 17) / 5.0) ** 2 + ((jj - 15) / 5.0) ** 2))

    def run(scheme, dt, T=43200.0):
        o = QgmTracOracle(dx=np.full((ny, nx), d), dy=np.full((ny, nx), d), dt=dt, SSH=ssh, c=2.7, g=9.81,
                          f=1.0e-4, time_scheme=scheme)
        return o.step(ssh, ssh, nstep=int(round(T / dt)))
    fine = run("rk4", 675.0)
    e4 = [np.abs(run("rk4", dt) - fine).max() for dt in (10800.0, 5400.0, 2700.0)]
    assert all(14.0 < e4[k] / e4[k + 1] < 18.0 for k in range(2))
    e2 = [np.abs(run("rk2", dt) - fine).max() for dt in (2700.0, 1350.0)]
    assert 3.5 < e2[0] / e2[1] < 4.5


# ---- tangent linear and adjoint (jax.jvp / vjp of step, jqgm.py:2141-2151)

def _tl_case(g, key, seed):
    from oracle.qg1l_trac import QgmTracTLAD
    rng = np.random.default_rng(seed)
    if key == "a":
        o = QgmTracTLAD(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                        time_scheme="Euler", Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC", mdt=g["a_mdt"])
        X0, Xb = g["a_X0"], g["a_Xb"]
    elif key == "b":
        o = QgmTracTLAD(dx=g["b_dx"], dy=g["b_dx"], dt=600.0, SSH=g["b_ssh"], c=2.5, g=9.81, f=1.0e-4,
                        time_scheme="rk2", Wbc=g["b_wbc"], Kdiffus_trac=5.0, bc_trac="dirichlet", advect_pv=False)
        X0, Xb = g["b_X0"], g["b_Xb"]
    elif key == "rk2obc":
        o = QgmTracTLAD(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                        time_scheme="rk2", Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC")
        X0, Xb = g["a_X0"], g["a_Xb"]
    elif key == "rk4":
        o = QgmTracTLAD(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                        time_scheme="rk4", Kdiffus_trac=10.0, bc_trac="OBC", mdt=g["a_mdt"])
        X0, Xb = g["a_X0"], g["a_Xb"]
    else:
        o = QgmTracTLAD(dx=g["c_dx"], dy=g["c_dx"], dt=900.0, SSH=g["c_ssh"], c=2.7, g=9.81, f=1.0e-4,
                        time_scheme="rk2", Kdiffus=15.0)
        X0, Xb = g["c_ssh"], g["c_hb"]
    X0 = np.nan_to_num(np.asarray(X0, dtype=np.float64))
    return o, X0, np.asarray(Xb, dtype=np.float64), rng


CASES = ["a", "b", "rk2obc", "rk4", "c"]


@pytest.mark.parametrize("key", CASES)
def test_trac_tangent_matches_central_differences(g, key):
    o, X0, Xb, rng = _tl_case(g, key, 31)
    d = rng.standard_normal(X0.shape) * np.abs(X0).max() * 1e-3
    tl = o.step_tgl(d, X0, Xb, 3)
    eps = 1e-4
    fd = (o.step(X0 + eps * d, Xb, 3) - o.step(X0 - eps * d, Xb, 3)) / (2 * eps)
    m = ~np.isnan(fd)
    assert np.all(tl[~m] == 0)
    err = np.abs(fd[m] - tl[m]).max() / np.abs(tl[m]).max()
    assert err <= 1e-7, err


@pytest.mark.parametrize("key", CASES)
def test_trac_adjoint_dot_product(g, key):
    o, X0, Xb, rng = _tl_case(g, key, 32)
    d = rng.standard_normal(X0.shape)
    y = rng.standard_normal(X0.shape)
    tl = o.step_tgl(d, X0, Xb, 3)
    ad = o.step_adj(y, X0, Xb, 3)
    lhs, rhs = float(np.sum(tl * y)), float(np.sum(d * ad))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
