"""The tracer point rules of the GPU kernels (vardyn_gb300/csrc/vd_qgtrac.cuh),
built for the host with g++, against the oracle's Qgm_trac restatement
(oracle/qg1l_trac.py, jqgm.py:1827-1866 and 1957-2006) on whole planes."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle.qg1l_trac import QgmTracOracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    so = str(tmp_path_factory.mktemp("qgtrac") / "qgtrac_points.so")
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "qgtrac_points_host.cpp")], check=True)
    L = ctypes.CDLL(so)
    P = ctypes.c_void_p
    L.trac_rhs_plane_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_double, P, P, P, P, P]
    L.trac_bc_plane_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, P, P, P, P, P, P, P]
    L.rk_combine_f64.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                 ctypes.POINTER(ctypes.c_double)]
    L.rk_combine_f64.restype = ctypes.c_double
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _model(land, K=7.0, obc=True, wbc=None):
    ny, nx = 23, 29
    ssh = np.zeros((ny, nx))
    if land:
        ssh[9:12, 12:16] = np.nan
    return QgmTracOracle(dx=np.full((ny, nx), 1.0e4), dy=np.full((ny, nx), 1.3e4), dt=800.0, SSH=ssh, c=2.7,
                         f=1.0e-4, Kdiffus_trac=K, bc_trac="OBC" if obc else "dirichlet", Wbc=wbc)


@pytest.mark.parametrize("land", [False, True])
@pytest.mark.parametrize("K", [None, 7.0])
def test_tracer_tendency_matches_oracle(lib, land, K):
    o = _model(land, K)
    rng = np.random.default_rng(5 + land)
    ny, nx = o.ny, o.nx
    u, v = rng.standard_normal((2, ny, nx)) * 0.3
    c = 1.0 + 0.2 * rng.standard_normal((ny, nx))
    c[o.ind0] = 0.0
    c[3, 4] = np.nan        # a NaN reaches the stencil of a few points: their tendency is 0
    var = np.stack([np.zeros((ny, nx)), c])
    want = o.rhs_state(u, v, None, None, var)[1]
    got = np.empty((ny, nx))
    mask = np.ascontiguousarray(o.mask, dtype=np.int8)
    lib.trac_rhs_plane_f64(ny, nx, o.dx, o.dy, 0 if K is None else 1, 0.0 if K is None else K, _p(mask),
                           _p(np.ascontiguousarray(u)), _p(np.ascontiguousarray(v)), _p(c), _p(got))
    assert np.array_equal(np.isnan(got), np.isnan(want)) and not np.isnan(got).any()
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()
    assert (got == 0).sum() == (want == 0).sum()


@pytest.mark.parametrize("obc", [True, False])
@pytest.mark.parametrize("custom_w", [False, True])
def test_tracer_boundary_update_matches_oracle(lib, obc, custom_w):
    ny, nx = 23, 29
    wbc = None
    if custom_w:
        wbc = np.zeros((ny, nx))
        wbc[:4, :] = np.linspace(0.9, 0.1, 4)[:, None]
        wbc[:, -3:] = 0.5
    o = _model(True, obc=obc, wbc=wbc)
    rng = np.random.default_rng(11 + obc + 2 * custom_w)
    u, v = rng.standard_normal((2, ny, nx)) * 0.3
    a, b, x = 1.0 + 0.1 * rng.standard_normal((3, ny, nx))
    want = o.bc(np.stack([np.zeros((ny, nx)), x]), np.stack([np.zeros((ny, nx)), a]), u, v,
                np.stack([np.zeros((ny, nx)), b]))[1]
    got = x.copy()
    mask = np.ascontiguousarray(o.mask, dtype=np.int8)
    W = np.ascontiguousarray(o.Wbc, dtype=np.float64)
    lib.trac_bc_plane_f64(ny, nx, o.dx, o.dy, o.dt, 1 if obc else 0, _p(mask), _p(np.ascontiguousarray(u)),
                          _p(np.ascontiguousarray(v)), _p(a), _p(b), _p(W), _p(got))
    assert np.abs(got - want).max() <= 1e-15
    assert not np.array_equal(got, x)


def test_rk4_combination_matches_oracle_order(lib):
    """The four RK4 combination modes give var0 + (k1 + 2 k2 + 2 k3 + k4)/6
    and the intermediate states var0 + k/2, var0 + k/2, var0 + k."""
    rng = np.random.default_rng(3)
    base, dt = 1.7, 600.0
    r = rng.standard_normal(4) * 1e-5
    acc = ctypes.c_double(0.0)
    s = [lib.rk_combine_f64(1, 0.5, dt, r[0], base, ctypes.byref(acc)),
         lib.rk_combine_f64(2, 0.5, dt, r[1], base, ctypes.byref(acc)),
         lib.rk_combine_f64(2, 1.0, dt, r[2], base, ctypes.byref(acc)),
         lib.rk_combine_f64(3, 1.0, dt, r[3], base, ctypes.byref(acc))]
    k = r * dt
    assert s[0] == base + 0.5 * k[0] and s[1] == base + 0.5 * k[1] and s[2] == base + k[2]
    assert s[3] == base + (k[0] + 2 * k[1] + 2 * k[2] + k[3]) / 6.0
    assert lib.rk_combine_f64(0, 1.0, dt, r[0], base, None) == base + dt * r[0]
