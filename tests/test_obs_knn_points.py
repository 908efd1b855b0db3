"""The observation neighbour search of the GPU kernel (vd_obs_knn.cuh),
built for the host with g++, against the oracle's restatements of both
reference operators (obsop.py:417-460 k-nearest; 197-219 with excluded ring
and mask points), inside, near and outside the grid."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import obsop as ob
from vardyn_gb300.obsop import l3_exclusion

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def knn(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    so = str(tmp_path_factory.mktemp("knn") / "obs_knn.so")
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "obs_knn_host.cpp")], check=True)
    f = ctypes.CDLL(so).obs_knn_host
    P = ctypes.c_void_p
    f.argtypes = [ctypes.c_longlong, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                  ctypes.c_int, ctypes.c_double, P, P, P]
    return f


def _run(knn, x, y, ny, nx, dx, dy, npix, excl):
    n = x.size
    idx = np.empty((n, 4), dtype=np.int64)
    w = np.empty((n, 4))
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    knn(n, p(x), p(y), ny, nx, dx / 1e3, dy / 1e3, npix, ob.dmax_km(dx, dy, npix),
        None if excl is None else p(excl), p(idx), p(w))
    return idx, w


def _dense(rows, cols, data, n, size):
    h = np.zeros((n, size))
    np.add.at(h, (rows, cols), data)
    return h


@pytest.mark.parametrize("npix", [1, 2, 4])
@pytest.mark.parametrize("rule", ["knn", "l3"])
def test_host_build_matches_oracle(knn, npix, rule):
    ny, nx, dx, dy = 22, 27, 4.0e3, 6.0e3
    rng = np.random.default_rng(npix + 10 * (rule == "l3"))
    n = 400
    x = rng.uniform(-25.0, nx * dx / 1e3 + 25.0, n)
    y = rng.uniform(-25.0, ny * dy / 1e3 + 25.0, n)
    mask = np.zeros((ny, nx), dtype=bool)
    mask[8:12, 10:16] = True
    excl = l3_exclusion(ny, nx, mask, mask_borders=True) if rule == "l3" else None
    idx, w = _run(knn, x, y, ny, nx, dx, dy, npix, excl)
    assert np.all(idx[:, npix:] == -1) and np.all(w[:, npix:] == 0)
    keep = idx >= 0
    rows = np.repeat(np.arange(n), 4).reshape(n, 4)
    got = _dense(rows[keep], idx[keep], w[keep], n, ny * nx)
    if rule == "l3":
        d, r, c = ob.sparse_op_l3(x, y, ny, nx, dx, dy, npix,
                                  ob.l3_excluded(ny, nx, dx, dy, mask, mask_borders=True))
    else:
        d, r, c = ob.sparse_op(x, y, ny, nx, dx, dy, npix)
    want = _dense(r, c, d, n, ny * nx)
    assert np.array_equal(got != 0, want != 0)
    assert np.abs(got - want).max() <= 1e-15
