"""Spectral Helmholtz oracle (restatement of helmholtz.py) against the
reference's own outputs, and the host-side recovery of (dx, dy, shift)
from a helm array used by the GPU drop-ins."""
import os

import numpy as np
import pytest

from oracle.helmholtz_dst import (compute_capacitance_matrices, compute_laplace_dstI, solve_helmholtz_dstI,
                                  solve_helmholtz_dstI_cmm)

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qg1l_golden.npz")
NX, NY, DX, DY, F0 = 40, 30, 2.0e3, 2.5e3, 1.0e-4


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def helm_of(g):
    return compute_laplace_dstI(NX, NY, DX, DY)[None, None] - F0 ** 2 * g["helm_lam"].reshape(1, 2, 1, 1)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_solve_matches_reference(g):
    assert rel(solve_helmholtz_dstI(g["helm_rhs"], helm_of(g)), g["helm_dst_sol"]) < 1e-13


def test_capacitance_matches_reference(g):
    cap = compute_capacitance_matrices(helm_of(g), g["helm_bx"], g["helm_by"])
    assert rel(cap, g["helm_cap"]) < 1e-12


def test_cmm_matches_reference(g):
    sol = solve_helmholtz_dstI_cmm(g["helm_rhs"], helm_of(g), g["helm_cap"], g["helm_bx"], g["helm_by"],
                                   g["helm_mask"])
    assert rel(sol, g["helm_cmm_sol"]) < 1e-13
    assert np.all(sol[..., g["helm_mask"] == 0] == 0)


def test_solve_inverts_five_point_operator():
    """Size-independent property: the interior of the solution satisfies
    (D_xx + D_yy - s) u = rhs with u = 0 on the walls."""
    rng = np.random.default_rng(3)
    nx, ny, dx, dy, s = 64, 48, 1.5, 0.7, 0.3
    rhs = rng.standard_normal((nx - 1, ny - 1))
    u = solve_helmholtz_dstI(rhs, compute_laplace_dstI(nx, ny, dx, dy) - s)
    w = np.zeros_like(u)
    w[1:-1, 1:-1] = u[1:-1, 1:-1]
    lap = ((w[2:, 1:-1] - 2 * w[1:-1, 1:-1] + w[:-2, 1:-1]) / dx ** 2
           + (w[1:-1, 2:] - 2 * w[1:-1, 1:-1] + w[1:-1, :-2]) / dy ** 2)
    assert rel(lap - s * w[1:-1, 1:-1], rhs) < 1e-12


def test_cmm_zero_on_boundary_points(g):
    """The capacitance correction makes the solution vanish at the
    irregular boundary points before masking."""
    helm = helm_of(g)
    sol = solve_helmholtz_dstI_cmm(g["helm_rhs"], helm, g["helm_cap"], g["helm_bx"], g["helm_by"],
                                   np.ones_like(g["helm_mask"]))
    assert np.abs(sol[..., g["helm_bx"] + 1, g["helm_by"] + 1]).max() < 1e-12 * np.abs(sol).max()


def test_infer_recovers_grid_and_shifts(g):
    from vardyn_gb300.helmholtz_dst import _infer
    nx, ny, dx, dy, shifts = _infer(helm_of(g))
    assert (nx, ny) == (NX, NY)
    assert abs(dx - DX) < 1e-9 * DX and abs(dy - DY) < 1e-9 * DY
    assert shifts[0] == 0.0 and abs(shifts[1] - F0 ** 2 * g["helm_lam"][1]) < 1e-12 * abs(shifts[1])


def test_infer_rejects_other_operators(g):
    from vardyn_gb300.helmholtz_dst import _infer
    h = helm_of(g).copy()
    h[0, 0, 5, 7] *= 1.01
    with pytest.raises(ValueError):
        _infer(h)
    with pytest.raises(ValueError):
        _infer(compute_laplace_dstI(NX, NY, DX, DY) + 1e-6)   # negative shift


def test_direct_masked_solve_equals_reference_capacitance_solve(g):
    """The direct sparse solve of the masked Dirichlet problem
    (oracle/helmholtz_masked.py, the checker of the multigrid) equals the
    reference's capacitance-matrix solution (golden vectors of helmholtz.py)
    on every ocean node: both solve the 5-point problem with u = 0 at the
    land points next to the ocean."""
    from oracle.helmholtz_masked import solve
    helm = helm_of(g)
    mask = g["helm_mask"]
    nl = helm.shape[-3]
    rhs = np.asarray(g["helm_rhs"])
    want = np.asarray(g["helm_cmm_sol"])
    inner = mask[..., 1:-1, 1:-1] if mask.ndim == 2 else mask.reshape(mask.shape[-2:])[1:-1, 1:-1]
    nx, ny = NX, NY
    shifts = [0.0] + [F0 ** 2 * float(g["helm_lam"][m]) for m in range(1, nl)]
    for m in range(nl):
        u = solve(nx - 1, ny - 1, DX, DY, shifts[m], inner, rhs.reshape((nl,) + rhs.shape[-2:])[m] * inner)
        w = want.reshape((nl,) + want.shape[-2:])[m][1:-1, 1:-1]
        assert np.abs(u - w * inner).max() <= 1e-11 * np.abs(w).max()
