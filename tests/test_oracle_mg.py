"""Masked multigrid Helmholtz oracle (restatement of the reference's
MG_Helmholtz) against a direct sparse solve of the same operator."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl

from oracle.helmholtz_mg import MGOracle, compute_nlevels


def case(n0=96, n1=64, seed=0):
    rng = np.random.default_rng(seed)
    mask = np.ones((n0, n1))
    mask[30:50, 20:35] = 0
    mask[:5, :7] = 0
    cu = 1.0 + 0.3 * rng.random((n0 + 1, n1))
    cv = 1.0 + 0.3 * rng.random((n0, n1 + 1))
    return rng, mask, cu, cv


def test_nlevels_matches_reference_rule():
    assert compute_nlevels(8) == 1
    assert compute_nlevels(96) == 4          # 96 = 32*3: 96/8 = 12 >= 8
    assert compute_nlevels(1024) == 8
    assert compute_nlevels(768) == 7


def test_pinv_bottom_converges_to_direct_solve():
    rng, mask, cu, cv = case()
    lam = np.array([1e-4, 5e-4])
    mg = MGOracle(1.0, 1.2, 96, 64, cu, cv, lam, mask=mask, niter_bottom=-1)
    rhs = rng.standard_normal((2, 96, 64)) * mask
    f = mg.solve(rhs)
    assert np.all(f[:, mask == 0] == 0)
    for b in range(2):
        A, i_s, j_s = mg.operator_matrix(b)
        x = spl.spsolve(A.tocsc(), rhs[b, i_s, j_s])
        assert np.linalg.norm(f[b, i_s, j_s] - x) / np.linalg.norm(x) < 1e-10


def test_jacobi_bottom_reduces_residual():
    rng, mask, cu, cv = case(seed=1)
    mg = MGOracle(1.0, 1.0, 96, 64, cu, cv, [1e-2], mask=mask, niter_bottom=20, max_ite=10)
    rhs = rng.standard_normal((1, 96, 64)) * mask
    f = mg.solve(rhs)
    from oracle.helmholtz_mg import residual
    r = residual(f, rhs, 1.0, 1.0, mg.masks[0], mg.cu[0], mg.cv[0], mg.lam)
    assert np.linalg.norm(r) < 1e-6 * np.linalg.norm(rhs)
